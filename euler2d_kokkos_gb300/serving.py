"""Batched execution and the serving loop on top of the e2d_batch C ABI.

run_batched      -- admit a set of solves (as many as the pool holds at a
                    time), advance them together until every one reaches its
                    t_end, refilling the pool as solves finish.
run_one_at_a_time -- the same solves as plain single-simulation runs, one
                    after the other (the baseline the batched mode is
                    compared with).
serve            -- continuous batching under open-loop Poisson arrivals:
                    requests arriving while others are on the GPU are
                    admitted as slots and pool bytes free up, every admitted
                    solve advances in the same per-iteration launch, and each
                    request's latency (arrival to completion) is recorded.

A FP32C solve whose state turns non-finite is stopped by the batch
(E2D_ENUMERIC; E2D_ETIMEOUT for a row-staging wait of the TMA variant that
gave up) without affecting the others.  With on_nonfinite="fp64" (the
default) it is admitted again from its initial state as an FP64 instance --
the bit-exact FP64 kernels, in the same batch -- and its latency runs from the
original arrival; "drop" records it in RunStats.failed instead.  FP32 arithmetic
can break down where FP64 does not: the reference's own single-precision build
(USE_DOUBLE off) also turns non-finite on such flows.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import PRECISION_FP32C, PRECISION_FP64, Batch, E2DError, HydroRun


@dataclass
class RunStats:
    cell_updates: int = 0
    seconds: float = 0.0
    solves: int = 0
    iterations: int = 0
    latencies: list = field(default_factory=list)
    tuning: tuple = ()
    failed: list = field(default_factory=list)     # indices of solves stopped for good
    escalated: list = field(default_factory=list)  # indices of FP32C solves re-run in FP64
    rejected: list = field(default_factory=list)   # indices of requests larger than the whole pool
    wasted_cell_updates: int = 0                   # updates of stopped solves (not in cell_updates)
    states: dict = field(default_factory=dict)     # serve(keep=...): index -> final state
    peak_live: int = 0                             # most solves on the GPU at once

    @property
    def gcell_per_s(self) -> float:
        return self.cell_updates / self.seconds / 1e9 if self.seconds > 0 else 0.0

    def percentiles(self):
        if not self.latencies:
            return {}
        a = np.asarray(self.latencies)
        return {"p50_s": float(np.percentile(a, 50)), "p95_s": float(np.percentile(a, 95)),
                "p99_s": float(np.percentile(a, 99)), "max_s": float(a.max()), "mean_s": float(a.mean())}


def _sync_device():
    try:
        import torch

        torch.cuda.synchronize()
    except Exception:
        pass


class _Reaper:
    """Completion handling shared by run_batched and serve: a solve that
    reached t_end is done; a stopped one is either queued again in FP64
    (policy "fp64", FP32C solves only) or recorded as failed."""

    def __init__(self, solves, stats, policy):
        if policy not in ("fp64", "drop"):
            raise ValueError("on_nonfinite must be 'fp64' or 'drop'")
        self.solves, self.stats, self.policy = solves, stats, policy
        self.fp64 = set()  # indices now running in FP64 after a FP32C failure

    def params(self, k):
        p = self.solves[k].params
        if k in self.fp64:
            p = p.copy()
            p.precision = PRECISION_FP64
            p.init()
        return p

    def reap(self, b, i, k):
        """State of instance i (solve k): None while it runs; True when it
        reached t_end; "retry" when it stopped and solve k is to be admitted
        again in FP64; False when it stopped for good.  Every outcome but
        None releases the instance."""
        _, ns, active, ok = b.poll(i)
        if ok and active:
            return None
        b.release(i)
        if ok:
            return True
        p = self.solves[k].params
        self.stats.wasted_cell_updates += ns * p.nx * p.ny
        if self.policy == "fp64" and p.precision == PRECISION_FP32C and k not in self.fp64:
            self.fp64.add(k)
            self.stats.escalated.append(k)
            return "retry"
        self.stats.failed.append(k)
        return False


def run_batched(solves, pool_bytes=64 << 30, iters_per_call=16, autotune=True, keep=None,
                on_nonfinite="fp64"):
    """Advance every solve to its t_end in one batch; solves that do not fit
    wait for room.  keep: optional set of indices whose final states are
    returned in `states`.  on_nonfinite: "fp64" or "drop" (module doc)."""
    stats = RunStats()
    reaper = _Reaper(solves, stats, on_nonfinite)
    states = {}
    with Batch(riemann="hllc", pool_bytes=pool_bytes, max_instances=max(len(solves), 1)) as b:
        pending = list(range(len(solves)))
        live = {}
        tuned = not autotune
        _sync_device()
        t0 = time.perf_counter()
        while pending or live:
            while pending:
                k = pending[0]
                try:
                    live[b.admit(reaper.params(k), solves[k].t_end, solves[k].u0)] = k
                except E2DError as e:
                    if e.status != 2 or not live:
                        raise
                    break
                pending.pop(0)
            if not tuned:
                b.autotune(2)
                tuned = True
            stats.peak_live = max(stats.peak_live, len(live))
            b.run(iters_per_call)
            stats.iterations += iters_per_call
            for i in list(live):
                k = live[i]
                if keep is not None and k in keep:
                    _, _, active, ok = b.poll(i)
                    if ok and not active:
                        states[k] = b.get_state(i)
                r = reaper.reap(b, i, k)
                if r is None:
                    continue
                live.pop(i)
                if r == "retry":
                    pending.insert(0, k)
                elif r:
                    stats.solves += 1
        stats.seconds = time.perf_counter() - t0
        stats.cell_updates = b.stats()[0] - stats.wasted_cell_updates
        stats.tuning = b.get_tuning()
    return stats, states


def _solve_alone(params, s, chunk):
    """One solve on its own handle to its t_end; returns the steps taken.
    A stopped run raises step_n's E2DError (its .nstep: the steps taken)."""
    with HydroRun(params, init_problem=s.u0 is None) as h:
        if s.u0 is not None:
            h.set_state(0, s.u0)
        t, ns = 0.0, 0
        while t < s.t_end:
            prev = ns
            t, ns, _ = h.step_n(chunk, s.t_end, t, ns, want_trace=False)
            if ns == prev:
                break
        h.current(ns)
        return ns


def run_one_at_a_time(solves, chunk=256, on_nonfinite="fp64"):
    """Each solve alone: its own simulation handle, the device time loop in
    graph-replayed chunks until t_end, its result read back.  A FP32C solve
    that stops (E2D_ENUMERIC / E2D_ETIMEOUT) is handled as run_batched
    handles it: re-run in FP64 ("fp64") or recorded as failed ("drop")."""
    stats = RunStats()
    reaper = _Reaper(solves, stats, on_nonfinite)
    _sync_device()
    t0 = time.perf_counter()
    for k, s in enumerate(solves):
        p = s.params
        while True:
            try:
                ns = _solve_alone(reaper.params(k), s, chunk)
            except E2DError as e:
                if e.status not in (3, 4):  # E2D_ENUMERIC, E2D_ETIMEOUT
                    raise
                stats.wasted_cell_updates += e.nstep * p.nx * p.ny
                if reaper.policy == "fp64" and p.precision == PRECISION_FP32C and k not in reaper.fp64:
                    reaper.fp64.add(k)
                    stats.escalated.append(k)
                    continue
                stats.failed.append(k)
                break
            stats.cell_updates += ns * p.nx * p.ny
            stats.solves += 1
            break
    stats.seconds = time.perf_counter() - t0
    return stats


def serve(solves, rate_per_s, pool_bytes=150 << 30, iters_per_call=8, seed=1, autotune=True,
          time_limit_s=None, on_nonfinite="fp64", keep=None):
    """Open-loop Poisson arrivals (rate_per_s) of `solves` in order; returns
    RunStats with per-request latencies and the aggregate throughput over
    the makespan.  on_nonfinite: "fp64" or "drop" (module doc).  keep:
    optional set of indices whose final states are returned in
    RunStats.states.  A request that does not fit even the empty pool is
    recorded in RunStats.rejected and never admitted."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, size=len(solves)))
    stats = RunStats()
    reaper = _Reaper(solves, stats, on_nonfinite)
    with Batch(riemann="hllc", pool_bytes=pool_bytes, max_instances=max(len(solves), 1)) as b:
        queue = []          # (index, arrival) waiting for admission
        live = {}           # instance id -> (index, arrival)
        nxt = 0
        tuned = not autotune
        _sync_device()
        t0 = time.perf_counter()
        while nxt < len(solves) or queue or live:
            now = time.perf_counter() - t0
            if time_limit_s is not None and now > time_limit_s:
                break
            while nxt < len(solves) and arrivals[nxt] <= now:
                queue.append((nxt, arrivals[nxt]))
                nxt += 1
            while queue:
                k, arr = queue[0]
                try:
                    i = b.admit(reaper.params(k), solves[k].t_end, solves[k].u0)
                except E2DError as e:
                    if e.status != 2:
                        raise
                    if live:
                        break  # no room: wait for completions
                    # the pool is empty and still too small: it never fits
                    stats.rejected.append(k)
                    queue.pop(0)
                    continue
                live[i] = (k, arr)
                queue.pop(0)
            if not live:
                # idle until the next arrival
                if nxt < len(solves):
                    time.sleep(max(0.0, min(arrivals[nxt] - (time.perf_counter() - t0), 0.05)))
                continue
            if not tuned and len(live) >= 4:
                b.autotune(2)
                tuned = True
            stats.peak_live = max(stats.peak_live, len(live))
            b.run(iters_per_call)
            stats.iterations += iters_per_call
            done_t = time.perf_counter() - t0
            for i in list(live):
                k, arr = live[i]
                if keep is not None and k in keep:
                    _, _, active, ok = b.poll(i)
                    if ok and not active:
                        stats.states[k] = b.get_state(i)
                r = reaper.reap(b, i, k)
                if r is None:
                    continue
                live.pop(i)
                if r == "retry":
                    queue.insert(0, (k, arr))
                elif r:
                    stats.latencies.append(done_t - arr)
                    stats.solves += 1
        stats.seconds = time.perf_counter() - t0
        stats.cell_updates = b.stats()[0] - stats.wasted_cell_updates
    return stats
