"""bench.py's batch summary on the CPU: the JSON it builds from the batched
and one-at-a-time runs, with the serving functions replaced by stand-ins
(no device work)."""
import importlib.util
import json
import os

import euler2d_kokkos_gb300 as e2d
from euler2d_kokkos_gb300 import serving

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_batch_summary_reports_reruns_and_failures(monkeypatch):
    bench = load_bench()

    def fake_batched(solves, **kw):
        st = serving.RunStats(cell_updates=10 ** 9, seconds=0.5, iterations=64, tuning=(4, [64, 64, 64]))
        st.solves, st.escalated, st.failed = len(solves) - 1, [3], [5]
        return st, {}

    def fake_alone(solves, **kw):
        st = serving.RunStats(cell_updates=10 ** 8, seconds=1.0)
        st.solves, st.escalated = len(solves), [1]
        return st

    monkeypatch.setattr(serving, "run_batched", fake_batched)
    monkeypatch.setattr(serving, "run_one_at_a_time", fake_alone)
    for fp64 in (False, True):
        out = bench.batch_summary(16, 4, fp64=fp64)
        json.dumps(out)
        assert out["value"] == 2.0 and out["batched_over_one_at_a_time"] == 20.0
        assert out["batched"]["rerun_fp64_after_nonfinite"] == [3] and out["batched"]["failed"] == [5]
        # one-at-a-time indices are mapped back to the batch's solve numbers
        idx = out["one_at_a_time"]["sample_indices"]
        assert len(idx) == 4 and idx == sorted(idx)
        assert out["one_at_a_time"]["rerun_fp64_after_nonfinite"] == [idx[1]]
        assert out["precision"] == ("fp64" if fp64 else "fp32c")
        assert out["instances"] == 16
