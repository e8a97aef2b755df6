"""Autotuner of the batched EM engine's work-item sizes.

    python -m fastem_gb300.autotune [--out fastem_gb300/tuning/batch_gb300.json]
                                    [--sweeps 6] [--repeats 2]

The batched engine (csrc/em_batch.cu) splits every fit's points into work
items per dimension class (d <= 4, 8, 16, 32): E-step items of 512 points
(fixed by the kernel), means items and covariance items of a per-class number
of points (fem_em_batch_tuning).  Small items give more CTAs for the few large
fits and more partial sums to reduce; large items the reverse.  The means and
covariance launches of a class are separate and timed separately (CUDA events,
fem_em_batch_timing_classes), so one run of the whole workload per candidate
size measures every class at once, and each class and phase takes its fastest
candidate.  The workload is the 512-fit batch of the bench (synth.em_batched,
seed 4: N log-uniform in [2e3, 2e5], d in {4, 8, 16, 32}, K in [2, 32]).

The table written holds the chosen sizes and every measurement behind them;
CudaBatchEM loads it by default.  Item sizes change the schedule and the order
of the FP32 item sums, not the sweep (tests/test_em_batch_gpu.py checks the
tuned engine against the FP64 oracle).
"""
import argparse
import json
import os
import time

import numpy as np

from . import synth
from .batch import CLASS_DIMS, TUNING_TABLE, CudaBatchEM
from .em import GaussianMixture

MEANS_CANDIDATES = (512, 1024, 2048, 4096, 8192)
COV_CANDIDATES = (1024, 2048, 4096, 8192)


def workload():
    fits = synth.em_batched()
    data = []
    for f in fits:
        X, _ = synth.kmeans_blobs(seed=f["seed"], n=f["n"], d=f["d"], k=f["k"])
        data.append((X, synth.dsquared_init(X, f["k"], seed=f["seed"] % 1000)))
    return data


def measure(data, tuning, sweeps, repeats, device=0):
    """per-class ms per sweep of the E-step, means and covariance launches"""
    shapes = [(X.shape[1], X.shape[0], len(init[0])) for X, init in data]
    packed = np.concatenate([X.reshape(-1) for X, _ in data])
    with CudaBatchEM(shapes, device=device, max_sweeps=sweeps, tuning=tuning) as B:
        B.SetParameters(sweeps, 0.0, 1e12)
        B.CopyPacked(packed)
        for i, (_, init) in enumerate(data):
            B.SetMixture(i, GaussianMixture(*init))
        B.TrainNoCopy()                      # warm-up
        best = None
        for _ in range(repeats):
            for i, (_, init) in enumerate(data):
                B.SetMixture(i, GaussianMixture(*init))
            B.EnableTiming(True)
            B.TrainNoCopy()
            tm = B.Timing()
            cl = tm["classes"]
            per = np.array([[cl[D][ph] for D in CLASS_DIMS] for ph in ("estep_ms", "means_ms", "cov_ms")])
            per /= max(1, tm["sweeps"])           # [phase][class], ms per sweep
            best = per if best is None else np.minimum(best, per)
            B.EnableTiming(False)
        return best


def tune(sweeps=6, repeats=2, device=0, log=print):
    data = workload()
    runs = []
    n = max(len(MEANS_CANDIDATES), len(COV_CANDIDATES))
    for i in range(n):
        m = MEANS_CANDIDATES[min(i, len(MEANS_CANDIDATES) - 1)]
        c = COV_CANDIDATES[min(i, len(COV_CANDIDATES) - 1)]
        t0 = time.perf_counter()
        per = measure(data, {"means_chunk": [m] * 4, "cov_chunk": [c] * 4}, sweeps, repeats, device)
        runs.append({"means_chunk": m, "cov_chunk": c, "ms_per_sweep": per.tolist()})
        log("means %5d cov %5d: means ms %s  cov ms %s  (%.1f s)" % (
            m, c, np.round(per[1], 3).tolist(), np.round(per[2], 3).tolist(), time.perf_counter() - t0))
    means, cov = [], []
    for cl in range(4):
        mbest = min(runs, key=lambda r: r["ms_per_sweep"][1][cl])
        cbest = min(runs, key=lambda r: r["ms_per_sweep"][2][cl])
        means.append(mbest["means_chunk"])
        cov.append(cbest["cov_chunk"])
    chosen = {"means_chunk": means, "cov_chunk": cov}
    check = measure(data, chosen, sweeps, repeats, device)
    default = measure(data, None, sweeps, repeats, device)
    return {
        "what": "points per means item and per covariance item of the batched EM engine, per dimension "
                "class (d <= 4, 8, 16, 32)",
        "workload": "512 fits (synth.em_batched, seed 4), %d sweeps per run, best of %d timed runs" % (sweeps,
                                                                                                    repeats),
        "classes": list(CLASS_DIMS),
        "means_chunk": means, "cov_chunk": cov,
        "ms_per_sweep_chosen": {"estep": check[0].tolist(), "means": check[1].tolist(), "cov": check[2].tolist()},
        "ms_per_sweep_default": {"estep": default[0].tolist(), "means": default[1].tolist(),
                                 "cov": default[2].tolist()},
        "candidates": runs,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=TUNING_TABLE)
    ap.add_argument("--sweeps", type=int, default=6)
    ap.add_argument("--repeats", type=int, default=2)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args()
    table = tune(a.sweeps, a.repeats, a.device)
    try:
        import torch
        table["gpu"] = torch.cuda.get_device_name(a.device)
    except Exception:
        pass
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(table, f, indent=1)
    print("wrote", a.out, "means", table["means_chunk"], "cov", table["cov_chunk"])


if __name__ == "__main__":
    main()
