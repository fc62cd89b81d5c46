"""Benchmark of the GB300 unsplit MUSCL-Hancock Godunov step.

Workload: the 4096x4096 blast (gamma 1.4, reflecting walls, rho = 1, p = 10
inside a disc of radius 0.125 at (0.5, 0.5), p = 0.1 outside, HLLC, CFL 0.8),
FP64.  One step = one time step of the device time loop (dt from the CFL
maximum of the current state, clamped at t_end; ghost fill, primitives,
slopes, trace, Riemann solves, conservative update).  The state (2 x 537 MB)
is larger than L2, so every step streams it from HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

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
BYTES_PER_CELL = {"fp64": 64}  # read U + write U, 4 variables


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=4096)
    ap.add_argument("--riemann", default="hllc", choices=["hllc", "hll", "approx"])
    ap.add_argument("--cpu-sample-steps", type=int, default=0,
                    help="steps of the CPU baseline sample (0: sized to ~15 s)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_params(e2d, nx, riemann):
    return e2d.make_params(nx, nx, problem="blast", riemann=riemann, gamma0=1.4, cfl=0.8,
                           slope_type=2.0, bc=(1, 1, 1, 1), blast_radius=0.125,
                           blast_center_x=0.5, blast_center_y=0.5, blast_density_in=1.0,
                           blast_density_out=1.0, blast_pressure_in=10.0, blast_pressure_out=0.1)


def config(nx, riemann, extra=None):
    c = {"workload": f"blast {nx}x{nx}, FP64, {riemann.upper()}, reflecting walls, CFL 0.8",
         "nx": nx, "ny": nx, "riemann": riemann, "precision": "fp64",
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


def ncu_traffic(kernel_prefix):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary, scaled to the benchmark's grid (profiles/*.json)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    try:
        d = json.load(open(path))
        e = d.get(kernel_prefix)
        return e
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
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(nx, riemann, steps, label_sample=True):
    """The oracle (reference FP64 algorithm, OpenMP) on the host cores."""
    from oracle import pyoracle as po

    p = po.make_params(nx, nx, gamma0=1.4, cfl=0.8, slope_type=2.0, bc=(1, 1, 1, 1), riemann=riemann)
    u0 = po.init_blast(p, radius=po.f32(0.125), cx=po.f32(0.5), cy=po.f32(0.5), d_in=1.0,
                       d_out=1.0, p_in=10.0, p_out=po.f32(0.1))
    threads = po.lib().orc_num_threads()
    if steps <= 0:
        # size the sample to roughly 15 s of CPU time
        t0 = time.perf_counter()
        po.run(p, u0, 1, 10.0)
        one = time.perf_counter() - t0
        steps = int(max(1, min(200, 15.0 / max(one, 1e-3))))
    t0 = time.perf_counter()
    _, _, _, ns = po.run(p, u0, steps, 10.0)
    el = time.perf_counter() - t0
    return {"value": nx * nx * ns / el / 1e9, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{ns} time steps of the {nx}x{nx} blast (oracle restatement of the "
                      f"reference's FP64 impl-0 step, OpenMP over {threads} threads), {el:.1f} s"}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    from oracle import pyoracle as po

    nx = args.nx
    p = po.make_params(nx, nx, gamma0=1.4, cfl=0.8, slope_type=2.0, bc=(1, 1, 1, 1), riemann="hllc")
    u = po.init_blast(p, radius=po.f32(0.125), cx=po.f32(0.5), cy=po.f32(0.5), d_in=1.0, d_out=1.0,
                      p_in=10.0, p_out=po.f32(0.1))
    u2 = u.copy()
    if args.warmup > 0:
        u, _, _, _ = po.run(p, u, args.warmup, 10.0)
        u2 = u.copy()
    threads = po.lib().orc_num_threads()
    t0 = time.perf_counter()
    _, dts, _, ns = po.run(p, u, args.steps, 10.0)
    el = time.perf_counter() - t0
    value = nx * nx * ns / el / 1e9
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0, "steps": ns,
            "warmup": args.warmup, "ms_per_step": el * 1e3 / max(ns, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": config(nx, "hllc", {"implementation": "CPU oracle: restatement of the "
                                          "reference's FP64 implementation-0 step (the reference "
                                          "runs HLLC whatever the riemann key says)"}),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": f"{ns} full time steps of the {nx}x{nx} blast"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
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
    p = workload_params(e2d, nx, args.riemann)
    h = e2d.HydroRun(p)
    stream = torch.cuda.ExternalStream(h.stream())
    t_end = 10.0
    # warm-up: W steps (graph capture happens here)
    t, ns = 0.0, 0
    if args.warmup > 0:
        t, ns, _ = h.step_n(args.warmup, t_end, t, ns)
    barrier()

    # timed region: exactly K steps, per-kernel CUDA events on the library's stream
    h.reset_kernel_times()
    h.set_profiling(True)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        barrier()
        ev0.record(stream)
        t, ns, _ = h.step_n(args.steps, t_end, t, ns)
        ev1.record(stream)
        barrier()
    ms = ev0.elapsed_time(ev1)
    kt = h.kernel_times()
    h.set_profiling(False)

    # the same K steps replayed from CUDA graphs (the production path)
    barrier()
    ev0.record(stream)
    t, ns, _ = h.step_n(args.steps, t_end, t, ns)
    ev1.record(stream)
    barrier()
    ms_graph = ev0.elapsed_time(ev1)
    ms_max = ms_graph
    if dist:
        tt = torch.tensor([ms_graph], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_max = float(tt.item())
    cells = nx * nx
    value = cells * args.steps * world / (ms_max / 1e3) / 1e9

    # end to end through the C ABI with host buffers: upload the initial
    # state from pinned memory, K steps, read the result back
    host_in = torch.empty((4, nx + 4, nx + 4), dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty_like(torch.from_numpy(host_in)).pin_memory().numpy()
    h0 = e2d.HydroRun(p)
    h0.get_state(0, host_in)
    h0.close()
    barrier()
    t0 = time.perf_counter()
    h.set_state(0, host_in)
    t2, ns2, _ = h.step_n(args.steps, t_end, 0.0, 0)
    h.get_state(ns2 % 2, host_out)
    e2e_s = time.perf_counter() - t0
    state_bytes = host_in.nbytes
    e2e = {"value": cells * ns2 / e2e_s / 1e9, "unit": METRIC,
           "h2d_bytes_per_step": state_bytes / max(ns2, 1),
           "d2h_bytes_per_step": (state_bytes + 8 * ns2) / max(ns2, 1),
           "path": "e2d_set_state + e2d_step_n + e2d_get_state from pinned host buffers"}

    k2_name = next((k for k in kt if k.startswith("k_flux_update")), None)
    peaks, peak_kind = measured_peaks()
    roof = None
    if k2_name:
        k2_ms, k2_n = kt[k2_name]
        avg_s = k2_ms / k2_n / 1e3
        alg_bytes = BYTES_PER_CELL["fp64"] * cells
        achieved = alg_bytes / avg_s / 1e9
        peak = float(peaks.get("hbm_gbs", HBM_FALLBACK_GBS))
        tr = ncu_traffic(k2_name.split("<")[0])
        traffic = None
        if tr and tr.get("bytes_per_cell"):
            traffic = tr["bytes_per_cell"] * cells
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": k2_name,
                "kernel_ms_avg": avg_s * 1e3, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6.8 TB/s",
                "note": "FP64 path: limited by the FP64 pipe, see fp64_pipe"}
        fp64 = json.load(open(os.path.join(ROOT, "profiles", "fp64_peak.json"))) \
            if os.path.exists(os.path.join(ROOT, "profiles", "fp64_peak.json")) else None
        if fp64:
            roof["fp64_pipe"] = {"dfma_peak_gops": fp64.get("dfma_gops"),
                                 "fp64_ops_per_cell": fp64.get("fp64_ops_per_cell")}
    kernels = {k: {"ms_total": v[0], "launches": v[1]} for k, v in kt.items()}
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "gb300",
            "config": config(nx, args.riemann),
            "ms_per_step_profiled": ms / args.steps,
            "kernels": kernels, "roofline": roof, "clocks": clocks.summary(), "e2e": e2e,
            "gpu_launches": int(sum(v[1] for v in kt.values())),
            "reference_formula_mcell_per_s": (nx + 4) ** 2 * args.steps * world / (ms_max / 1e3) / 1e6}
    h.close()
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(nx, "hllc", args.cpu_sample_steps)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
