"""Benchmark of the GB300 unsplit MUSCL-Hancock Godunov step.

Headline workload (default): the 4096x4096 blast in FP64 -- gamma 1.4,
reflecting walls, rho = 1, p = 10 inside a disc of radius 0.125 at
(0.5, 0.5), p = 0.1 outside, HLLC, CFL 0.8.  One step = one time step of the
device time loop (dt from the CFL maximum of the current state, clamped at
t_end; ghost fill, primitives, slopes, trace, Riemann solves, conservative
update).  The state (2 x 537 MB) is larger than L2, so every step streams it
from HBM.

Secondary (in the same JSON line, key "fp32c"): the 8192x8192 four-quadrant
Riemann problem (Lax-Liu 3 split at 0.5, absorbing walls, HLLC, CFL 0.8) in
the FP32 compensated mode, with its relative L1 density error against the
FP64 path (which is bit-identical to the reference) on the same 8192x8192
grid after the same number of steps as the timed run, and at 1024x1024 to
t = 0.3.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--precision fp64|fp32c] [--problem blast|four_quadrant] [--nx N]

Prints one JSON line.  `--impl reference` times the reference algorithm on
the host cores instead: the CPU oracle (a restatement of the reference's own
FP64 code, OpenMP over all cores) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Gcell-updates/s"
HBM_FALLBACK_GBS = 6800.0
BYTES_PER_CELL = {"fp64": 64, "fp32c": 64, "fp64_fast": 64}  # read + write of the 4 conserved variables
BLAST = dict(blast_radius=0.125, blast_center_x=0.5, blast_center_y=0.5, blast_density_in=1.0,
             blast_density_out=1.0, blast_pressure_in=10.0, blast_pressure_out=0.1)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32c", "fp64_fast"])
    ap.add_argument("--problem", default=None, choices=["blast", "four_quadrant"])
    ap.add_argument("--nx", type=int, default=None)
    ap.add_argument("--riemann", default="hllc", choices=["hllc", "hll", "approx"])
    ap.add_argument("--cpu-sample-steps", type=int, default=0,
                    help="steps of the CPU baseline sample (0: sized to ~15 s)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--mode", default="step", choices=["step", "batch", "serve", "c3", "f64tiles", "fp64peak"],
                    help="step: one grid (default); batch: 512 mixed solves batched vs one at a "
                         "time; serve: Poisson arrivals into the batched loop; c3: the 8192^2 "
                         "four-quadrant problem to t = 0.3 in FP32C, in FP64 and in FP64 from a perturbed "
                         "initial state (about 40 min at 8192^2, 5 min at 4096^2); f64tiles: the FP64 "
                         "step at every tile shape, fused and as two launches; fp64peak: the FP64 "
                         "operation rates of this GPU")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--sample", type=int, default=0,
                    help="solves timed one at a time in --mode batch (0: all of them)")
    ap.add_argument("--rates", default="", help="arrival rates (solves/s) for serve mode, comma-separated")
    ap.add_argument("--serve-seconds", type=float, default=20.0)
    ap.add_argument("--c3-nx", type=int, default=8192, help="grid side of --mode c3")
    ap.add_argument("--repeat", type=int, default=0, help="--mode f64tiles: interleaved repeats of the HLLC forms")
    a = ap.parse_args()
    if a.problem is None:
        a.problem = "four_quadrant" if a.precision == "fp32c" else "blast"
    if a.nx is None:
        a.nx = 4096 if a.problem == "blast" else 8192
    return a


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def workload_params(e2d, problem, nx, riemann, precision):
    prec = {"fp64": e2d.PRECISION_FP64, "fp32c": e2d.PRECISION_FP32C,
            "fp64_fast": e2d.PRECISION_FP64_FAST}[precision]
    if problem == "blast":
        return e2d.make_params(nx, nx, problem="blast", riemann=riemann, gamma0=1.4, cfl=0.8,
                               slope_type=2.0, bc=(1, 1, 1, 1), precision=prec, **BLAST)
    return e2d.make_params(nx, nx, problem="four_quadrant", riemann=riemann, gamma0=1.4, cfl=0.8,
                           slope_type=2.0, bc=(2, 2, 2, 2), precision=prec, fq_split_x=0.5,
                           fq_split_y=0.5)


def workload_name(problem, nx, riemann, precision):
    if problem == "blast":
        return f"blast {nx}x{nx}, {precision.upper()}, {riemann.upper()}, reflecting walls, CFL 0.8"
    return (f"four-quadrant (Lax-Liu 3, split 0.5) {nx}x{nx}, {precision.upper()}, {riemann.upper()}, "
            f"absorbing walls, CFL 0.8")


def config(problem, nx, riemann, precision, extra=None):
    c = {"workload": workload_name(problem, nx, riemann, precision), "nx": nx, "ny": nx,
         "riemann": riemann, "precision": precision,
         "l2": f"state {4 * (nx + 4) ** 2 * 8 / 1e6:.0f} MB per array > 129 MB L2 (no flush needed)",
         "parallelism": "replicas"}
    if extra:
        c.update(extra)
    return c


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            return json.load(open(path)), "measured"
        except Exception:
            pass
    return {"hbm_gbs": HBM_FALLBACK_GBS}, "fallback"


def ncu_traffic(kernel):
    """DRAM bytes per cell of a kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    try:
        return json.load(open(path)).get(kernel)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


def oracle_setup(problem, nx, riemann):
    from oracle import pyoracle as po

    if problem == "blast":
        p = po.make_params(nx, nx, gamma0=1.4, cfl=0.8, slope_type=2.0, bc=(1, 1, 1, 1), riemann=riemann)
        u0 = po.init_blast(p, radius=po.f32(0.125), cx=po.f32(0.5), cy=po.f32(0.5), d_in=1.0,
                           d_out=1.0, p_in=10.0, p_out=po.f32(0.1))
    else:
        p = po.make_params(nx, nx, gamma0=1.4, cfl=0.8, slope_type=2.0, bc=(2, 2, 2, 2), riemann=riemann)
        u0 = po.init_four_quadrant(p, xt=po.f32(0.5), yt=po.f32(0.5))
    return po, p, u0


def cpu_baseline(problem, nx, steps):
    """The oracle (reference FP64 algorithm, OpenMP) on the host cores."""
    po, p, u0 = oracle_setup(problem, nx, "hllc")
    threads = po.lib().orc_num_threads()
    if steps <= 0:  # size the sample to roughly 15 s of CPU time
        t0 = time.perf_counter()
        po.run(p, u0, 1, 10.0)
        one = time.perf_counter() - t0
        steps = int(max(1, min(200, 15.0 / max(one, 1e-3))))
    t0 = time.perf_counter()
    _, _, _, ns = po.run(p, u0, steps, 10.0)
    el = time.perf_counter() - t0
    return {"value": nx * nx * ns / el / 1e9, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{ns} time steps of the {nx}x{nx} {problem} (oracle restatement of the "
                      f"reference's FP64 implementation-0 step, OpenMP over {threads} threads), {el:.1f} s"}


def run_reference_arm(args, rank):
    if rank != 0:
        return
    po, p, u = oracle_setup(args.problem, args.nx, "hllc")
    t0 = time.perf_counter()
    if args.warmup > 0:
        u, _, _, _ = po.run(p, u, args.warmup, 10.0)
    per_step = (time.perf_counter() - t0) / max(args.warmup, 1)
    # K steps, or as many as fit in about two minutes of host time
    steps = max(1, min(args.steps, int(120.0 / max(per_step, 1e-9)))) if args.warmup > 0 else args.steps
    threads = po.lib().orc_num_threads()
    t0 = time.perf_counter()
    _, dts, _, ns = po.run(p, u, steps, 10.0)
    el = time.perf_counter() - t0
    value = args.nx * args.nx * ns / el / 1e9
    _, world, _ = dist_env()
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": ns,
            "warmup": args.warmup, "ms_per_step": el * 1e3 / max(ns, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": config(args.problem, args.nx, "hllc", "fp64",
                             {"implementation": "CPU oracle: restatement of the reference's FP64 "
                                                "implementation-0 step, bit-identical to it (the "
                                                "reference itself runs HLLC whatever the riemann key says)"}),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": f"{ns} full time steps of the {args.nx}x{args.nx} {args.problem} "
                                       f"(of {args.steps} asked; capped at ~2 min of host time)"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def max_over_ranks(dist, x: float) -> float:
    """The largest x over all ranks (the job's time is its slowest rank's);
    x itself without a process group."""
    if not dist:
        return x
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measure(e2d, torch, args, precision, problem, nx, steps, warmup, local, barrier, dist,
            with_e2e=True, with_clocks=True, riemann=None, env=None):
    saved = {k: os.environ.get(k) for k in (env or {})}
    os.environ.update(env or {})  # read by the library when a handle is created
    try:
        return _measure(e2d, torch, args, precision, problem, nx, steps, warmup, local, barrier, dist,
                        with_e2e, with_clocks, riemann)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _measure(e2d, torch, args, precision, problem, nx, steps, warmup, local, barrier, dist,
             with_e2e, with_clocks, riemann):
    p = workload_params(e2d, problem, nx, riemann or args.riemann, precision)
    h = e2d.HydroRun(p)
    stream = torch.cuda.ExternalStream(h.stream())
    t_end = 10.0
    t, ns = 0.0, 0
    if warmup > 0:
        t, ns, _ = h.step_n(warmup, t_end, t, ns)
    barrier()
    # timed region 1: exactly K steps with per-kernel CUDA events on the library's stream
    h.reset_kernel_times()
    h.set_profiling(True)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local) if with_clocks else None
    if sampler:
        sampler.__enter__()
    barrier()
    ev0.record(stream)
    t, ns, _ = h.step_n(steps, t_end, t, ns)
    ev1.record(stream)
    barrier()
    if sampler:
        sampler.__exit__(None, None, None)
    ms_prof = ev0.elapsed_time(ev1)
    kt = h.kernel_times()
    h.set_profiling(False)
    # timed region 2: the same K steps replayed from CUDA graphs (the production path)
    barrier()
    ev0.record(stream)
    t, ns, _ = h.step_n(steps, t_end, t, ns)
    ev1.record(stream)
    barrier()
    ms_max = max_over_ranks(dist, ev0.elapsed_time(ev1))
    out = {"ms": ms_max, "ms_profiled": ms_prof, "kernels": kt,
           "clocks": sampler.summary() if sampler else None}
    if with_e2e:
        # end to end through the C ABI with host buffers: upload the initial
        # state from pinned memory, K steps, read the result back
        host_in = torch.empty((4, nx + 4, nx + 4), dtype=torch.float64, pin_memory=True).numpy()
        host_out = torch.empty((4, nx + 4, nx + 4), dtype=torch.float64, pin_memory=True).numpy()
        h0 = e2d.HydroRun(p)
        h0.get_state(0, host_in)
        h0.get_state(0, host_out)  # both buffers touched before the timed region
        h0.close()
        barrier()
        t0 = time.perf_counter()
        h.set_state(0, host_in)
        t1 = time.perf_counter()
        _, ns2, _ = h.step_n(steps, t_end, 0.0, 0)
        t2 = time.perf_counter()
        h.get_state(ns2 % 2, host_out)
        t3 = time.perf_counter()
        e2e_s = max_over_ranks(dist, t3 - t0)
        world = dist.get_world_size() if dist else 1
        out["e2e"] = {"value": nx * nx * ns2 * world / e2e_s / 1e9, "unit": METRIC,
                      "h2d_bytes_per_step": host_in.nbytes / max(ns2, 1),
                      "d2h_bytes_per_step": (host_out.nbytes + 8 * ns2) / max(ns2, 1),
                      "path": "e2d_set_state + e2d_step_n + e2d_get_state from pinned host buffers, "
                              f"{ns2} steps per call",
                      "seconds": {"set_state": t1 - t0, "step_n": t2 - t1, "get_state": t3 - t2}}
    h.close()
    return out


def roofline(kt, precision, cells, prefix):
    name = next((k for k in kt if k.startswith(prefix)), None)
    if not name:
        return None
    peaks, kind = measured_peaks()
    k_ms, k_n = kt[name]
    avg_s = k_ms / k_n / 1e3
    alg = BYTES_PER_CELL[precision] * cells
    achieved = alg / avg_s / 1e9
    peak = float(peaks.get("hbm_gbs", HBM_FALLBACK_GBS))
    tr = ncu_traffic(name)
    r = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
         "traffic": (tr["bytes_per_cell"] * cells) if tr and tr.get("bytes_per_cell") else None,
         "kernel": name, "kernel_ms_avg": avg_s * 1e3,
         "algorithmic_bytes_per_launch": alg,
         "peak_source": ("of measured (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured"
                         else "of fallback 6.8 TB/s")}
    if tr:
        r["traffic_source"] = tr.get("source")
    return r


# FP64 operations of the fused FP64 step (k_step_f64 in
# euler2d_kokkos_gb300/csrc/e2d_fp64.cu), counted from its source, by kind:
# "addmul" (adds, subtracts, multiplies), "fma", "div", "sqrt" and "max"
# (fmax and FP64 comparisons).  Each kind is weighted by its measured cost
# in FMA-rate cycles (FMA rate / its rate: on GB300 adds and multiplies run
# at ~0.84 of the FMA rate, a division or a square root costs ~9 FMAs).
# Limiter min/max, sign tests, cut-offs against positive constants and the
# exact scalings by 0.5 and 2 run on the integer pipe and are not counted.
F64_OPS = {
    # stage 2, per cell of the tile and of its 1-cell ring: 8 limited slopes
    # (3 subtractions each, f64x::slope_limited) and the trace sources
    # (trace_sources: 10 products and 10 sums; dpx / r and dpy / r)
    "slopes_trace": {"addmul": 24 + 20, "div": 2},
    # face_pair for the 4 variables of one direction: s0 * dtd, then
    # q - h + sx and q + h + sx
    "faces_dir": {"addmul": 4 * 5},
    # stage 3, one solve plus the 4 products by dt/dx
    "hllc": {"addmul": 51 + 4, "div": 6, "sqrt": 2},
    "hll": {"addmul": 64 + 4, "div": 3, "sqrt": 2},
    # epilogue per cell: the update (4 x 4 sums), primitives (7 + 3
    # divisions), the CFL term (6 + a division and a square root), and
    # fmax / comparisons (the running maximum, the dx / dy power-of-two
    # tests, the density test, the block fold's shuffles, ~6)
    "epilogue": {"addmul": 16 + 7 + 6, "div": 3 + 1, "sqrt": 1, "max": 6},
}
# The opt-in fast forms (precision fp64_fast, *_fast in e2d_fp64_blocks.cuh):
# FMAs, and one reciprocal per denominator (rcp_nr: a hardware estimate on
# the MUFU unit and two Newton steps, 4 FMAs) in place of the divisions.
F64_OPS_FAST = {
    "slopes_trace": {"addmul": 24 + 6, "fma": 12},
    "faces_dir": {"fma": 4 * 3},
    "hllc": {"addmul": 39, "fma": 27, "sqrt": 2},
    "hll": {"addmul": 42, "fma": 26, "sqrt": 2},
    "epilogue": {"addmul": 28, "fma": 7, "sqrt": 1, "max": 4},
}
F64_TILES = {-1: (32, 32), 0: (32, 32), 1: (32, 16), 2: (32, 31), 3: (32, 15)}  # E2D_F64_TILE -> shape


def tile_shape(tile, fast=False):
    """(TX, TY) of the fused FP64 step for an E2D_F64_TILE value (the fast
    forms exist for 32 x 16 and 32 x 32)."""
    if fast:
        return (32, 16) if tile == 1 else (32, 32)
    return F64_TILES.get(tile, (32, 32))


def fp64_ops_per_cell(riemann, tile=-1, fast=False):
    """FP64 operations per cell-update of the fused step by kind, for a tile
    shape: per tile, (TX+2)(TY+2)-4 slope/trace evaluations, 2 TX TY + 2 TX
    + 2 TY face-pair directions, (TX+1) TY + TX (TY+1) solves and TX TY
    epilogues.  None for the iterative approx solver."""
    ops = F64_OPS_FAST if fast else F64_OPS
    if riemann not in ops:
        return None
    tx, ty = tile_shape(tile, fast)
    n = {"slopes_trace": (tx + 2) * (ty + 2) - 4, "faces_dir": 2 * tx * ty + 2 * tx + 2 * ty,
         riemann: (tx + 1) * ty + tx * (ty + 1), "epilogue": tx * ty}
    tot = {"addmul": 0.0, "fma": 0.0, "div": 0.0, "sqrt": 0.0, "max": 0.0}
    for part, cnt in n.items():
        for kind, v in ops[part].items():
            tot[kind] += cnt * v / (tx * ty)
    return tot


_FP64_RATES = None


def fp64_pipe_counts(kernel):
    """FP64-pipe instructions per cell of a kernel from the committed ncu
    capture (profiles/fp64_pipe.json), or None."""
    path = os.path.join(ROOT, "profiles", "fp64_pipe.json")
    if not os.path.exists(path):
        return None
    return json.load(open(path)).get(kernel)


def fp64_pipe_info(e2d, riemann, kernel_ms, cells, tile=-1, fast=False):
    """FP64-pipe roofline of the fused step, live: the probe's measured rates
    (e2d_fp64_rates, this run), the source-counted operations per cell in FMA
    equivalents, and the fraction of the FMA peak the kernel sustained."""
    global _FP64_RATES
    if _FP64_RATES is None:
        _FP64_RATES = e2d.fp64_rates()
    r = _FP64_RATES
    ops = fp64_ops_per_cell(riemann, tile, fast)
    out = {"rates_gops": r, "peak_gops": r["fma"], "unit": "G FP64 FMA-equivalent ops/s",
           "peak_source": "e2d_fp64_rates probe in this run (8 chains/thread, 8x256 threads/SM, CUDA events)"}
    if not ops:
        return out
    cost = {"fma": 1.0, "addmul": r["fma"] / min(r["add"], r["mul"]), "div": r["fma"] / r["div"],
            "sqrt": r["fma"] / r["sqrt"], "max": r["fma"] / r["max"]}
    per_cell = sum(ops[k] * cost[k] for k in ops)
    achieved = per_cell * cells / (kernel_ms * 1e-3) / 1e9
    out.update({"ops_per_cell": ops, "fma_equivalent_per_cell": per_cell,
                "cost_in_fma": {k: cost[k] for k in ("addmul", "div", "sqrt", "max")},
                "achieved_gops": achieved, "frac_algorithmic": achieved / r["fma"],
                "ops_source": "counted from k_step_f64's source (bench.py F64_OPS), divisions and square "
                              "roots weighted by their measured cost"})
    # the instructions the FP64 pipe actually executes per cell (one ncu
    # capture of this kernel; the division and square-root sequences and the
    # compiler add to the source count) at the live cell rate: the pipe's
    # busy fraction, as ncu's sm__pipe_fp64_cycles_active measures it
    tx, ty = tile_shape(tile, fast)
    ic = fp64_pipe_counts(f"k_step_f64<{riemann}>" + (" fast" if fast else "") + f" {tx}x{ty}")
    if ic:
        inst = ic["fp64_pipe_inst_per_cell"] * cells / (kernel_ms * 1e-3) / 1e9
        out.update({"fp64_pipe_inst_per_cell": ic["fp64_pipe_inst_per_cell"], "achieved_inst_gops": inst,
                    "frac": inst / r["fma"], "ncu_busy_pct_same_kernel": ic.get("fp64_pipe_busy_pct"),
                    "inst_source": ic.get("source")})
    return out


def l1_check(e2d, nx, t_end, problem="four_quadrant"):
    """FP32C vs FP64 (bit-identical to the reference) on the problem at nx^2
    to t_end: relative L1 of density, FP64 accumulation."""
    hs = {}
    for prec in ("fp64", "fp32c"):
        h = e2d.HydroRun(workload_params(e2d, problem, nx, "hllc", prec))
        t, ns = 0.0, 0
        while t < t_end and ns < 1_000_000:
            t, ns, tr = h.step_n(512, t_end, t, ns)
            if len(tr) == 0:
                break
        hs[prec] = (h, t, ns)
    (h64, t64, n64), (h32, t32, n32) = hs["fp64"], hs["fp32c"]
    d, r = h32.l1_diff(n32 % 2, h64, n64 % 2, e2d.ID)
    mass0 = None
    res = {"grid": f"{nx}x{nx}", "t_end": t_end, "steps_fp64": n64, "steps_fp32c": n32,
           "rel_l1_density_vs_fp64": d / r, "oracle": "FP64 GPU path (bit-identical to the reference)"}
    for h, _, _ in hs.values():
        h.close()
    return res


def l1_steps(e2d, problem, nx, steps, precs=("fp64", "fp32c")):
    """FP32C (or another precision) vs FP64 (bit-identical to the reference)
    on the bench's own workload: the same initial state advanced `steps`
    steps of the device time loop at nx^2; relative L1 of density (FP64
    accumulation) and the largest relative difference of the dt sequences."""
    out = {}
    for prec in precs:
        h = e2d.HydroRun(workload_params(e2d, problem, nx, "hllc", prec))
        t, ns, tr = h.step_n(steps, 10.0, 0.0, 0)
        out[prec] = (h, t, ns, np.asarray(tr))
    (h64, t64, n64, tr64), (h32, t32, n32, tr32) = out[precs[0]], out[precs[1]]
    d, r = h32.l1_diff(n32 % 2, h64, n64 % 2, e2d.ID)  # on the device, FP64 sums
    h32.close()
    h64.close()
    n = min(len(tr64), len(tr32))
    return {"grid": f"{nx}x{nx}", "steps": n32, "steps_fp64": n64, "t_fp32c": t32, "t_fp64": t64,
            "rel_l1_density_vs_fp64": d / r,
            "dt_max_rel_diff": float(np.max(np.abs(tr32[:n] - tr64[:n]) / tr64[:n])) if n else None,
            "oracle": "FP64 GPU path (bit-identical to the reference), same initial state and step count"}


def fp64_l1_of(e2d, solve, got):
    """Relative L1 density error of a batched FP32C result against the FP64
    path (bit-identical to the reference) run to the same t_end."""
    p64 = solve.params.copy()
    p64.precision = e2d.PRECISION_FP64
    with e2d.HydroRun(p64.init(), init_problem=solve.u0 is None) as h:
        if solve.u0 is not None:
            h.set_state(0, solve.u0)
        t, ns = 0.0, 0
        while t < solve.t_end:
            prev = ns
            t, ns, _ = h.step_n(512, solve.t_end, t, ns, want_trace=False)
            if ns == prev:
                break
        ref = h.current(ns)
    a, r = got[0, 2:-2, 2:-2], ref[0, 2:-2, 2:-2]
    return float(np.abs(a - r).sum() / np.abs(r).sum())


BATCH_WORKLOAD = ("mixed solves: blasts (pressure ratio 10..1e4) and four-quadrant problems, sides "
                  "log-uniform 64..1024 (multiples of 16), t_end U[0.05,0.25], HLLC, CFL 0.8, seed 0")
SERVE_WORKLOAD = ("Poisson arrivals of blasts, four-quadrant problems and shocked bubbles (Mach 1.2..3, "
                  "density ratio 0.1..10), grids 64^2..2048^2, t_end U[0.05,0.25], 150 GB pool, HLLC, CFL 0.8")


def size_quartiles(solves):
    """Grid cells (nx * ny) of a set of solves: min, quartiles, max."""
    c = np.array([s.cells for s in solves], dtype=np.float64)
    return [int(x) for x in np.percentile(c, [0, 25, 50, 75, 100])]


def batch_summary(instances, sample, fp64=False):
    """Mixed 64^2-1024^2 blasts and four-quadrant problems (seed 0), each to
    its own t_end: one batched run of all of them against the same kind of
    solves run one at a time, HLLC, CFL 0.8; FP32 compensated (with the L1
    error of the smallest sampled solves against the FP64 path), or FP64
    (each result bit-identical to the single FP64 path)."""
    import euler2d_kokkos_gb300 as e2d
    from euler2d_kokkos_gb300 import serving, workloads

    prec = e2d.PRECISION_FP64 if fp64 else e2d.PRECISION_FP32C
    solves = workloads.mixed_batch(instances, seed=0, precision=prec)
    # the one-at-a-time sample: every k-th solve in order of grid size, so
    # that it spans the mix's size distribution (sample >= instances: all)
    by_size = sorted(range(len(solves)), key=lambda k: (solves[k].cells, k))
    stride = max(1, len(solves) // sample)
    sample_idx = sorted(by_size[stride // 2::stride][:sample]) if sample < len(solves) else list(range(len(solves)))
    # accuracy: the smallest sampled solves against the FP64 path
    small = [] if fp64 else sorted(sample_idx, key=lambda k: solves[k].cells)[:3]
    bstats, states = serving.run_batched(solves, pool_bytes=64 << 30, keep=set(small))
    seq = serving.run_one_at_a_time([solves[k] for k in sample_idx])
    l1 = [fp64_l1_of(e2d, solves[k], states[k]) for k in small if k in states]
    out_l1 = {"bitwise_equal_to_single_fp64_path": "tests/test_gpu_batch.py"} if fp64 else \
        {"rel_l1_density_vs_fp64": l1}
    return {"workload": f"{len(solves)} {BATCH_WORKLOAD}", "instances": len(solves),
            "precision": "fp64" if fp64 else "fp32c",
            "cells_total": sum(s.cells for s in solves),
            "tuning": {"variant": bstats.tuning[0], "strip_h_per_class": bstats.tuning[1]},
            "value": bstats.gcell_per_s, "unit": METRIC,
            "batched": {"value": bstats.gcell_per_s, "seconds": bstats.seconds,
                        "cell_updates": bstats.cell_updates, "launch_iterations": bstats.iterations,
                        "rerun_fp64_after_nonfinite": list(bstats.escalated), "failed": list(bstats.failed)},
            "one_at_a_time": {"value": seq.gcell_per_s, "seconds": seq.seconds, "solves": seq.solves,
                              "cell_updates": seq.cell_updates,
                              "rerun_fp64_after_nonfinite": [sample_idx[k] for k in seq.escalated],
                              "failed": [sample_idx[k] for k in seq.failed],
                              "sample": (f"all {len(solves)} solves" if len(sample_idx) == len(solves) else
                                         f"{len(sample_idx)} of the {len(solves)} solves: every {stride}th in "
                                         f"order of grid size"),
                              "sample_indices": sample_idx,
                              "cells_quartiles_sample": size_quartiles([solves[k] for k in sample_idx]),
                              "cells_quartiles_mix": size_quartiles(solves)},
            "batched_over_one_at_a_time": bstats.gcell_per_s / seq.gcell_per_s if seq.gcell_per_s else None,
            **out_l1}


def serve_summary(rates, seconds, max_requests):
    """Open-loop Poisson arrivals of mixed solves (the batch mix plus shocked
    bubbles, grids 64^2..2048^2) into a 150 GB pool; one entry per arrival
    rate with latency percentiles and aggregate throughput."""
    from euler2d_kokkos_gb300 import serving, workloads

    results = []
    for rate in rates:
        n = max(8, int(rate * seconds))
        solves = workloads.mixed_batch(min(n, max_requests), seed=1, max_side=2048, bubbles=True)
        st = serving.serve(solves, rate, pool_bytes=150 << 30, time_limit_s=seconds * 4)
        tag = lambda k: f"{k}: {solves[k].kind} {solves[k].params.nx}x{solves[k].params.ny}"
        results.append({"rate_per_s": rate, "requests": len(solves), "completed": st.solves,
                        "failed_nonfinite": [tag(k) for k in st.failed],
                        "rerun_fp64_after_nonfinite": [tag(k) for k in st.escalated],
                        "wasted_cell_updates": st.wasted_cell_updates,
                        "value": st.gcell_per_s, "seconds": st.seconds, **st.percentiles()})
    return results


def mode_line(value, mode, config_, extra):
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": 0, "warmup": 0,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (compensated hi/lo state, FP64 dt)", "data": "synthetic", "impl": "gb300",
            "mode": mode, "config": config_}
    line.update(extra)
    return line


def batch_mode(args):
    """The C4 batches with every solve also run one at a time (--sample
    defaults to all of them here)."""
    sample = args.instances if args.sample <= 0 else args.sample
    with ClockSampler(0) as clocks:
        b = batch_summary(args.instances, sample)
        b64 = batch_summary(max(8, args.instances // 8), max(8, args.instances // 8) if args.sample <= 0
                            else max(2, args.sample // 3), fp64=True)
    line = mode_line(b["value"], "batch", {"workload": b["workload"], "instances": b["instances"],
                                           "cells_total": b["cells_total"], "tuning": b["tuning"]},
                     {**{k: b[k] for k in ("batched", "one_at_a_time", "batched_over_one_at_a_time",
                                           "rel_l1_density_vs_fp64")}, "fp64": b64})
    line["steps"] = b["batched"]["launch_iterations"]
    line["ms_per_step"] = b["batched"]["seconds"] * 1e3 / max(line["steps"], 1)
    line["clocks"] = clocks.summary()
    print(json.dumps(line), flush=True)


def serve_mode(args):
    rates = [float(r) for r in args.rates.split(",") if r] or [4.0, 8.0, 16.0, 24.0, 32.0]
    with ClockSampler(0) as clocks:
        sweep = serve_summary(rates, args.serve_seconds, args.instances)
    best = max(sweep, key=lambda r: r["value"])
    line = mode_line(best["value"], "serve", {"workload": SERVE_WORKLOAD}, {"sweep": sweep})
    line["clocks"] = clocks.summary()
    print(json.dumps(line), flush=True)


def c3_mode(args):
    """C3 at its full size: the four-quadrant problem (--c3-nx, 8192^2 by
    default) run to t = 0.3 in FP32C and in FP64 (bit-identical to the
    reference, the transitive oracle), plus a control: FP64 again from the
    initial state multiplied by 1 + 1e-7 N(0, 1) (seed 0).  Reports the
    relative L1 of density of FP32C and of the control against FP64: the
    control measures how much this flow amplifies a perturbation of FP32's
    size by t = 0.3."""
    import torch

    import euler2d_kokkos_gb300 as e2d

    nx, t_end = args.c3_nx, 0.3
    runs = {}
    for prec in ("fp32c", "fp64", "fp64_control"):
        h = e2d.HydroRun(workload_params(e2d, "four_quadrant", nx, "hllc", "fp32c" if prec == "fp32c" else "fp64"))
        if prec == "fp64_control":
            u = h.U
            u = u * (1.0 + 1e-7 * np.random.default_rng(0).standard_normal(u.shape))
            h.set_state(0, u)
            h.set_state(1, u)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t, ns = 0.0, 0
        while t < t_end:
            prev = ns
            t, ns, _ = h.step_n(1024, t_end, t, ns, want_trace=False)
            if ns == prev:
                break
        torch.cuda.synchronize()
        runs[prec] = (h, t, ns, time.perf_counter() - t0)
    (h32, t32, n32, s32), (h64, t64, n64, s64) = runs["fp32c"], runs["fp64"]
    hc, tc, nc, sc = runs["fp64_control"]
    d, r = h32.l1_diff(n32 % 2, h64, n64 % 2, e2d.ID)
    dc, rc = hc.l1_diff(nc % 2, h64, n64 % 2, e2d.ID)
    line = mode_line(nx * nx * n32 / s32 / 1e9, "c3",
                     {"workload": workload_name("four_quadrant", nx, "hllc", "fp32c") + f", to t = {t_end}"},
                     {"fp32c": {"steps": n32, "t": t32, "seconds": s32, "gcell_per_s": nx * nx * n32 / s32 / 1e9},
                      "fp64": {"steps": n64, "t": t64, "seconds": s64, "gcell_per_s": nx * nx * n64 / s64 / 1e9},
                      "rel_l1_density_fp32c_vs_fp64": d / r,
                      "rel_l1_density_control_vs_fp64": dc / rc,
                      "control": "FP64 from the initial state times 1 + 1e-7 N(0,1)",
                      "oracle": "FP64 GPU path (bit-identical to the reference)"})
    for h, *_ in runs.values():
        h.close()
    print(json.dumps(line), flush=True)


def f64tiles_mode(args):
    """The FP64 blast (--nx, HLLC and HLL) at every fused-step tile shape and
    as two launches per step, CUDA events on the library's stream.  With
    --repeat R the HLLC forms are measured R times in turn instead and the
    line gives each form's median (timings of the forms interleave, so that
    drifts of the GPU affect them alike)."""
    import torch

    import euler2d_kokkos_gb300 as e2d

    nx = args.nx
    cells = nx * nx
    bar = torch.cuda.synchronize
    rows = []
    if args.repeat > 0:
        forms = [("fused 32x16", {"E2D_F64_TILE": "1"}), ("fused 32x32", {"E2D_F64_TILE": "0"}),
                 ("two launches 32x32", {"E2D_F64_SPLIT": "1", "E2D_F64_TILE": "0"})]
        got = {f: [] for f, _ in forms}
        with ClockSampler(0) as clocks:
            for _ in range(args.repeat):
                for label, env in forms:
                    m = measure(e2d, torch, args, "fp64", "blast", nx, args.steps, args.warmup, 0, bar, None,
                                with_e2e=False, with_clocks=False, riemann="hllc", env=env)
                    got[label].append(m["ms"] / args.steps)
        rows = [{"form": f, "ms_per_step_median": float(np.median(v)), "ms_per_step": v,
                 "gcell_per_s_median": cells / (float(np.median(v)) / 1e3) / 1e9} for f, v in got.items()]
        print(json.dumps({"metric": METRIC, "mode": "f64tiles", "repeat": args.repeat, "steps": args.steps,
                          "config": config("blast", nx, "hllc", "fp64"), "rows": rows,
                          "clocks": clocks.summary()}), flush=True)
        return
    with ClockSampler(0) as clocks:
        for rs in ("hllc", "hll"):
            for label, prec, env in [
                    ("fused 32x32 (default)", "fp64", {"E2D_F64_TILE": "0"}),
                    ("fused 32x16", "fp64", {"E2D_F64_TILE": "1"}),
                    ("fused 32x31", "fp64", {"E2D_F64_TILE": "2"}), ("fused 32x15", "fp64", {"E2D_F64_TILE": "3"}),
                    ("two launches 32x32", "fp64", {"E2D_F64_SPLIT": "1", "E2D_F64_TILE": "0"}),
                    ("fast, fused 32x32 (default)", "fp64_fast", {"E2D_F64_TILE": "0"}),
                    ("fast, fused 32x16", "fp64_fast", {"E2D_F64_TILE": "1"})]:
                m = measure(e2d, torch, args, prec, "blast", nx, args.steps, args.warmup, 0, bar, None,
                            with_e2e=False, with_clocks=False, riemann=rs, env=env)
                kt = {k: round(v[0] / v[1], 4) for k, v in m["kernels"].items()}
                row = {"riemann": rs, "form": label, "ms_per_step": m["ms"] / args.steps,
                       "gcell_per_s": cells * args.steps / (m["ms"] / 1e3) / 1e9, "kernel_ms_avg": kt}
                if "fused" in label:
                    k = next(k for k in kt if k.startswith("k_step_f64"))
                    row["fp64_pipe"] = fp64_pipe_info(e2d, rs, kt[k], cells, int(env["E2D_F64_TILE"]),
                                                      fast=prec == "fp64_fast")
                rows.append(row)
    line = {"metric": METRIC, "mode": "f64tiles", "config": config("blast", nx, "hllc/hll", "fp64"),
            "steps": args.steps, "rows": rows, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def fp64peak_mode(args):
    import euler2d_kokkos_gb300 as e2d

    with ClockSampler(0) as clocks:
        rates = [e2d.fp64_rates() for _ in range(3)]
    best = {k: max(r[k] for r in rates) for k in rates[0]}
    print(json.dumps({"mode": "fp64peak", "unit": "G FP64 operations/s", "rates": best, "runs": rates,
                      "clocks": clocks.summary()}), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return
    if args.mode == "batch":
        if rank == 0:
            batch_mode(args)
        return
    if args.mode == "serve":
        if rank == 0:
            serve_mode(args)
        return
    if args.mode == "c3":
        if rank == 0:
            c3_mode(args)
        return
    if args.mode in ("f64tiles", "fp64peak"):
        if rank == 0:
            (f64tiles_mode if args.mode == "f64tiles" else fp64peak_mode)(args)
        return

    import torch

    import euler2d_kokkos_gb300 as e2d

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as td

        td.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist = td

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    nx = args.nx
    cells = nx * nx
    m = measure(e2d, torch, args, args.precision, args.problem, nx, args.steps, args.warmup, local,
                barrier, dist)
    value = cells * args.steps * world / (m["ms"] / 1e3) / 1e9
    kt = m["kernels"]
    f64 = args.precision in ("fp64", "fp64_fast")
    prefix = "k_step_f64" if f64 else "k_step_f32c"
    roof = roofline(kt, args.precision, cells, prefix)
    if roof and f64:
        roof["note"] = "the FP64 step is bound by GB300's FP64 pipe, not HBM: see fp64_pipe"
        roof["fp64_pipe"] = fp64_pipe_info(e2d, args.riemann, roof["kernel_ms_avg"], cells,
                                           int(os.environ.get("E2D_F64_TILE", "-1")),
                                           fast=args.precision == "fp64_fast")
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if f64 else "f32 (compensated hi/lo state, FP64 dt)",
            "data": "synthetic", "impl": "gb300",
            "config": config(args.problem, nx, args.riemann, args.precision),
            "ms_per_step_profiled": m["ms_profiled"] / args.steps,
            "kernels": {k: {"ms_total": v[0], "launches": v[1]} for k, v in kt.items()},
            "roofline": roof, "clocks": m["clocks"], "e2e": m["e2e"],
            "gpu_launches": int(sum(v[1] for v in kt.values())),
            "reference_formula_mcell_per_s": (nx + 4) ** 2 * args.steps * world / (m["ms"] / 1e3) / 1e6}

    if not args.no_secondary and args.precision == "fp64" and rank == 0:  # the default line
        # the FP32 compensated mode on the four-quadrant problem at 8192^2
        s = measure(e2d, torch, args, "fp32c", "four_quadrant", 8192, args.steps, args.warmup, local,
                    barrier, None, with_e2e=False, with_clocks=False)
        sc = 8192 * 8192
        line["fp32c"] = {
            "config": config("four_quadrant", 8192, args.riemann, "fp32c"),
            "value": sc * args.steps / (s["ms"] / 1e3) / 1e9, "unit": METRIC,
            "ms_per_step": s["ms"] / args.steps,
            "roofline": roofline(s["kernels"], "fp32c", sc, "k_step_f32c"),
            "accuracy": {**l1_steps(e2d, "four_quadrant", 8192, args.steps),
                         "to_t_0.3_at_1024": l1_check(e2d, 1024, 0.3)}}
        # the C2 blast in the FP32 compensated mode, with its error against FP64
        sb = measure(e2d, torch, args, "fp32c", args.problem, nx, args.steps, args.warmup, local,
                     barrier, None, with_e2e=False, with_clocks=False)
        line["fp32c_blast"] = {
            "config": config(args.problem, nx, args.riemann, "fp32c"),
            "value": cells * args.steps / (sb["ms"] / 1e3) / 1e9, "unit": METRIC,
            "ms_per_step": sb["ms"] / args.steps,
            "roofline": roofline(sb["kernels"], "fp32c", cells, "k_step_f32c"),
            "accuracy": {**l1_steps(e2d, args.problem, nx, args.steps),
                         "to_t_0.05_at_1024": l1_check(e2d, 1024, 0.05, args.problem)}}
        # C2 also names the HLL solver: the same FP64 blast with it
        hl = measure(e2d, torch, args, "fp64", args.problem, nx, args.steps, args.warmup, local,
                     barrier, None, with_e2e=False, with_clocks=False, riemann="hll")
        rh = roofline(hl["kernels"], "fp64", cells, "k_step_f64")
        if rh:
            rh["fp64_pipe"] = fp64_pipe_info(e2d, "hll", rh["kernel_ms_avg"], cells)
        line["hll"] = {"config": config(args.problem, nx, "hll", "fp64"),
                       "value": cells * args.steps / (hl["ms"] / 1e3) / 1e9, "unit": METRIC,
                       "ms_per_step": hl["ms"] / args.steps, "roofline": rh}
        # the same FP64 step as two launches (fill + flux/update; the
        # primitives array round-trips through HBM), against the fused step
        tl = measure(e2d, torch, args, "fp64", args.problem, nx, args.steps, args.warmup, local,
                     barrier, None, with_e2e=False, with_clocks=False, env={"E2D_F64_SPLIT": "1"})
        line["fp64_two_launch"] = {
            "config": config(args.problem, nx, args.riemann, "fp64"),
            "value": cells * args.steps / (tl["ms"] / 1e3) / 1e9, "unit": METRIC,
            "ms_per_step": tl["ms"] / args.steps,
            "kernels": {k: {"ms_total": v[0], "launches": v[1]} for k, v in tl["kernels"].items()},
            "fused_over_two_launch": (tl["ms"] / m["ms"])}
        # the opt-in fast FP64 forms (FMAs, shared reciprocals; not
        # bit-identical) on the same workload, with their error against the
        # bit-exact FP64 path on this grid after the same steps
        fa = measure(e2d, torch, args, "fp64_fast", args.problem, nx, args.steps, args.warmup, local,
                     barrier, None, with_e2e=False, with_clocks=False)
        rf = roofline(fa["kernels"], "fp64_fast", cells, "k_step_f64")
        if rf:
            rf["fp64_pipe"] = fp64_pipe_info(e2d, args.riemann, rf["kernel_ms_avg"], cells, fast=True)
        line["fp64_fast"] = {
            "config": config(args.problem, nx, args.riemann, "fp64_fast"),
            "value": cells * args.steps / (fa["ms"] / 1e3) / 1e9, "unit": METRIC,
            "ms_per_step": fa["ms"] / args.steps, "roofline": rf,
            "accuracy": l1_steps(e2d, args.problem, nx, args.steps, precs=("fp64", "fp64_fast")),
            "tolerance": "dt within 1e-12 relative, relative L1 <= 1e-10 (tests/test_gpu_fp64_fast.py)"}
        # batched mixed solves against one at a time, and one loaded serving point
        line["batch"] = batch_summary(512, 64)
        line["batch_fp64"] = batch_summary(64, 16, fp64=True)
        line["serve"] = {"workload": SERVE_WORKLOAD, "sweep": serve_summary([32.0], 10.0, 320)}

    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.problem, min(nx, 4096), args.cpu_sample_steps)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
