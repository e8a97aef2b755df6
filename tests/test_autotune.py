"""CPU tests of the batched engine's work-item autotuner (fastem_gb300/autotune.py):
the choice per dimension class and phase from measured timings, and the table
format that CudaBatchEM loads.  The timings are supplied by a stand-in for the
GPU measurement."""
import json

import numpy as np

from fastem_gb300 import autotune, batch


def fake_measure(data, tuning, sweeps, repeats, device=0):
    """[phase][class] ms per sweep.  For a candidate run (one size for every
    class) the means phase of class c is fastest at means candidate c % 5 and
    the covariance phase at covariance candidate (c + 1) % 4; the run of the
    chosen sizes and the library defaults (tuning None) get flat timings."""
    per = np.ones((3, 4))
    if tuning is None:
        return per * 99.0
    ms, cs = tuning["means_chunk"], tuning["cov_chunk"]
    if len(set(ms)) == 1 and len(set(cs)) == 1:
        for c in range(4):
            per[1, c] = 1.0 + abs(autotune.MEANS_CANDIDATES.index(ms[0]) - c % 5)
            per[2, c] = 1.0 + abs(autotune.COV_CANDIDATES.index(cs[0]) - (c + 1) % 4)
    return per


def test_autotune_picks_fastest_per_class_and_phase(monkeypatch, tmp_path):
    monkeypatch.setattr(autotune, "workload", lambda: None)
    monkeypatch.setattr(autotune, "measure", fake_measure)
    t = autotune.tune(sweeps=1, repeats=1, log=lambda *a: None)
    assert t["means_chunk"] == [autotune.MEANS_CANDIDATES[c % 5] for c in range(4)]
    assert t["cov_chunk"] == [autotune.COV_CANDIDATES[(c + 1) % 4] for c in range(4)]
    assert t["classes"] == list(batch.CLASS_DIMS)
    # every candidate run is recorded with its timings
    assert len(t["candidates"]) == max(len(autotune.MEANS_CANDIDATES), len(autotune.COV_CANDIDATES))
    assert all(np.shape(r["ms_per_sweep"]) == (3, 4) for r in t["candidates"])
    # the table round-trips through the loader CudaBatchEM uses
    p = tmp_path / "table.json"
    p.write_text(json.dumps(t))
    assert batch.load_tuning(str(p)) == {"means_chunk": t["means_chunk"], "cov_chunk": t["cov_chunk"]}


def test_candidates_are_valid_item_sizes():
    # the engine accepts multiples of 128 in [256, 16384] (fem_em_batch_tuning)
    for v in autotune.MEANS_CANDIDATES + autotune.COV_CANDIDATES:
        assert v % 128 == 0 and 256 <= v <= 16384


def test_missing_table_means_library_defaults(tmp_path):
    assert batch.load_tuning(str(tmp_path / "absent.json")) is None
