"""Host logic of the serving drivers, on the CPU: what happens to a solve
that a batch stops with E2D_ENUMERIC, against a stand-in batch (no device
work)."""
import pytest

import euler2d_kokkos_gb300 as e2d
from euler2d_kokkos_gb300 import serving
from euler2d_kokkos_gb300 import workloads as W


class FakeBatch:
    """poll/release of e2d.Batch over a table id -> (t, nstep, active, ok)."""

    def __init__(self, table):
        self.table = dict(table)
        self.released = []

    def poll(self, i):
        return self.table[i]

    def release(self, i):
        self.released.append(i)


def solves(precision):
    return W.mixed_batch(2, seed=3, max_side=128, precision=precision)


def test_running_solve_is_left_alone():
    st = serving.RunStats()
    r = serving._Reaper(solves(e2d.PRECISION_FP32C), st, "fp64")
    b = FakeBatch({7: (0.01, 5, True, True)})
    assert r.reap(b, 7, 0) is None and b.released == []


def test_finished_solve_is_released():
    st = serving.RunStats()
    r = serving._Reaper(solves(e2d.PRECISION_FP32C), st, "fp64")
    b = FakeBatch({7: (0.1, 50, False, True)})
    assert r.reap(b, 7, 1) is True and b.released == [7]
    assert st.failed == [] and st.escalated == [] and st.wasted_cell_updates == 0


def test_fp32c_failure_is_rerun_once_in_fp64():
    sv = solves(e2d.PRECISION_FP32C)
    st = serving.RunStats()
    r = serving._Reaper(sv, st, "fp64")
    p = sv[1].params
    b = FakeBatch({3: (0.02, 9, True, False), 4: (0.01, 4, True, False)})
    assert r.reap(b, 3, 1) == "retry"
    assert st.escalated == [1] and st.wasted_cell_updates == 9 * p.nx * p.ny
    p64 = r.params(1)
    assert p64.precision == e2d.PRECISION_FP64 and p.precision == e2d.PRECISION_FP32C
    assert (p64.nx, p64.ny, p64.problemType) == (p.nx, p.ny, p.problemType)
    # the FP64 run stops too: recorded, not re-queued again
    assert r.reap(b, 4, 1) is False
    assert st.failed == [1] and st.escalated == [1] and b.released == [3, 4]
    assert st.wasted_cell_updates == 13 * p.nx * p.ny
    assert r.params(0) is sv[0].params


def test_fp64_failure_and_drop_policy_are_not_rerun():
    for prec, policy in ((e2d.PRECISION_FP64, "fp64"), (e2d.PRECISION_FP32C, "drop")):
        st = serving.RunStats()
        r = serving._Reaper(solves(prec), st, policy)
        assert r.reap(FakeBatch({0: (0.0, 1, True, False)}), 0, 0) is False
        assert st.failed == [0] and st.escalated == []


def test_unknown_policy_is_refused():
    with pytest.raises(ValueError):
        serving._Reaper([], serving.RunStats(), "retry")


class FakeRun:
    """HydroRun stand-in: FP32C runs stop with E2D_ENUMERIC after 5 steps,
    FP64 runs reach t_end in 7."""

    def __init__(self, params, init_problem=True):
        self.p = params

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def set_state(self, which, u):
        pass

    def step_n(self, n, t_end, t, nstep, want_trace=True):
        if self.p.precision == e2d.PRECISION_FP32C:
            err = e2d.E2DError(3, "step_n")
            err.t, err.nstep = 0.01, nstep + 5
            raise err
        return t_end, nstep + 7, None

    def current(self, nstep):
        return None


def test_one_at_a_time_applies_the_same_policy(monkeypatch):
    monkeypatch.setattr(serving, "HydroRun", FakeRun)
    sv = solves(e2d.PRECISION_FP32C)
    cells = [s.params.nx * s.params.ny for s in sv]
    st = serving.run_one_at_a_time(sv)
    assert st.solves == 2 and st.escalated == [0, 1] and st.failed == []
    assert st.cell_updates == 7 * sum(cells) and st.wasted_cell_updates == 5 * sum(cells)
    st = serving.run_one_at_a_time(sv, on_nonfinite="drop")
    assert st.solves == 0 and st.failed == [0, 1] and st.escalated == []
    st = serving.run_one_at_a_time(solves(e2d.PRECISION_FP64))
    assert st.solves == 2 and st.escalated == [] and st.wasted_cell_updates == 0


class FullPoolBatch:
    """e2d.Batch stand-in whose pool never has room: admit always raises
    E2D_ENOMEM, as e2d_batch_admit does for a solve larger than the pool."""

    def __init__(self, **kw):
        self.admits = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def admit(self, params, t_end, u0=None):
        self.admits += 1
        raise e2d.E2DError(2, "e2d_batch_admit")

    def stats(self):
        return (0, 0)


def test_serve_rejects_a_request_the_empty_pool_cannot_hold(monkeypatch):
    """With nothing live, E2D_ENOMEM means the request never fits: serve()
    records it and goes on instead of waiting for completions that cannot
    come (no time limit is given, so a wait would never end)."""
    monkeypatch.setattr(serving, "Batch", FullPoolBatch)
    sv = solves(e2d.PRECISION_FP32C)
    st = serving.serve(sv, rate_per_s=1e6, autotune=False)
    assert st.rejected == [0, 1] and st.solves == 0 and st.latencies == []


def test_run_batched_raises_on_a_request_the_empty_pool_cannot_hold(monkeypatch):
    monkeypatch.setattr(serving, "Batch", FullPoolBatch)
    with pytest.raises(e2d.E2DError) as ei:
        serving.run_batched(solves(e2d.PRECISION_FP32C), autotune=False)
    assert ei.value.status == 2
