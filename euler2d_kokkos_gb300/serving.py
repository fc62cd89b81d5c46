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
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import Batch, E2DError, HydroRun


@dataclass
class RunStats:
    cell_updates: int = 0
    seconds: float = 0.0
    solves: int = 0
    iterations: int = 0
    latencies: list = field(default_factory=list)
    tuning: tuple = ()

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


def run_batched(solves, pool_bytes=64 << 30, iters_per_call=16, autotune=True, keep=None):
    """Advance every solve to its t_end in one batch; solves that do not fit
    wait for room.  keep: optional set of indices whose final states are
    returned in `states`."""
    stats = RunStats()
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
                    live[b.admit(solves[k].params, solves[k].t_end, solves[k].u0)] = k
                except E2DError as e:
                    if e.status != 2 or not live:
                        raise
                    break
                pending.pop(0)
            if not tuned:
                b.autotune(2)
                tuned = True
            b.run(iters_per_call)
            stats.iterations += iters_per_call
            for i in list(live):
                t, ns, active = b.query(i)
                if not active:
                    k = live.pop(i)
                    if keep is not None and k in keep:
                        states[k] = b.get_state(i)
                    b.release(i)
                    stats.solves += 1
        stats.seconds = time.perf_counter() - t0
        stats.cell_updates = b.stats()[0]
        stats.tuning = b.get_tuning()
    return stats, states


def run_one_at_a_time(solves, chunk=256):
    """Each solve alone: its own simulation handle, the device time loop in
    graph-replayed chunks until t_end, its result read back."""
    stats = RunStats()
    _sync_device()
    t0 = time.perf_counter()
    for s in solves:
        with HydroRun(s.params, init_problem=s.u0 is None) as h:
            if s.u0 is not None:
                h.set_state(0, s.u0)
            t, ns = 0.0, 0
            while t < s.t_end:
                prev = ns
                t, ns, _ = h.step_n(chunk, s.t_end, t, ns, want_trace=False)
                if ns == prev:
                    break
            h.current(ns)
            stats.cell_updates += ns * s.params.nx * s.params.ny
            stats.solves += 1
    stats.seconds = time.perf_counter() - t0
    return stats


def serve(solves, rate_per_s, pool_bytes=150 << 30, iters_per_call=8, seed=1, autotune=True,
          time_limit_s=None):
    """Open-loop Poisson arrivals (rate_per_s) of `solves` in order; returns
    RunStats with per-request latencies and the aggregate throughput over
    the makespan."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, size=len(solves)))
    stats = RunStats()
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
                    i = b.admit(solves[k].params, solves[k].t_end, solves[k].u0)
                except E2DError as e:
                    if e.status != 2:
                        raise
                    break  # no room: wait for completions
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
            b.run(iters_per_call)
            stats.iterations += iters_per_call
            done_t = time.perf_counter() - t0
            for i in list(live):
                _, _, active = b.query(i)
                if not active:
                    k, arr = live.pop(i)
                    stats.latencies.append(done_t - arr)
                    b.release(i)
                    stats.solves += 1
        stats.seconds = time.perf_counter() - t0
        stats.cell_updates = b.stats()[0]
    return stats
