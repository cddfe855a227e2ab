#!/usr/bin/env python
"""Particle-steps/s of the GB300 SPH hot path on the 3-D dam break.

One step = one leap-frog iteration (half kick, cell hash + radix sort,
pass A, pass B, update) of the whole particle system, in FP64.  The default
workload is the 3-D dam break: a 0.6 x 0.3 x 0.6 m water block (1,687,500
particles, dx = 4 mm) in a 1.6 x 0.6 x 1.0 m box with 3 layers of wall
particles (1,024,008); its state (~1 GB) is far larger than the 129 MB L2.

Prints one JSON line.  `value` is timed on the device with inputs resident
in HBM; `e2e` times the C-ABI call a host that owns the particle arrays
makes (sph_step_host: pinned host x, v, rho, e in and out every step);
`roofline` reports the dominant kernel against the measured HBM copy
bandwidth and, because this path is FP64-bound on GB300, `roofline_fp64`
against a measured FP64 FMA rate.  `--impl reference` times the oracle's
OpenMP build (the CPU restatement of the reference) on the host cores.

Two more objects ride on the same line (N=1 only): `batched`, the 256-system
2-D ensemble in one batch context (FP32 pair loops, FP64 state) against the
same batch in FP64 and the plain FP64 path one system at a time, with the
relative L2 of its fields against FP64 at t_end; and `serving`, a Poisson
request stream continuously batched on the device with its p50/p99
time-to-solution.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s"
# algorithmic bytes per particle-step of each stage, FP64 (pair passes count
# each particle's own compulsory reads/writes; neighbour reads are served
# from L1/L2): pass A reads x, v, m, rho, h, type and writes drho, div v,
# strain; pass B reads x, v, m, rho, h, type, c, strain and writes a, de;
# the update reads v, rho, e, Prev, rates, x, h, c, div v and writes x, v,
# rho, e, Prev, displacement.  Hash and reorder traffic earns no credit.
ALGO_BYTES = {
    2: {"pass_a": 108, "pass_b": 124, "update": 232, "hash": 0, "permute": 0},
    3: {"pass_a": 164, "pass_b": 188, "update": 296, "hash": 0, "permute": 0},
}
# the same per stage for the mixed-precision form in 3-D (FP32 pair-loop
# reads and writes; the update adds the FP32 mirrors it writes)
ALGO_BYTES_MIXED_3D = {"pass_a": 84, "pass_b": 96, "update": 292, "hash": 0, "permute": 0}
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="dam_break_3d",
                    choices=["dam_break_3d", "dam_break_2d", "gate_2d"])
    ap.add_argument("--dx", type=float, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=4,
                    help="full-size oracle steps of the CPU baseline sample (about 10 s on 16 cores)")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--precision", choices=["fp64", "mixed", "df64"], default="fp64",
                    help="precision of the main (timed) run")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-system ensemble")
    ap.add_argument("--no-serving", action="store_true", help="skip the served request stream")
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--long-run", type=int, default=2000, metavar="STEPS",
                    help="run the 3-D dam break STEPS steps in FP64, mixed and DF64 from one state and "
                         "state each field's error against FP64 (2,000 steps: about a minute; 0 = off)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the 2-D dam break (1,000 steps, FP64) and the elastic-gate window")
    ap.add_argument("--gate-window", type=int, default=500,
                    help="steps of the elastic-gate window (FP64 and mixed)")
    ap.add_argument("--lanes", type=int, default=1, choices=[1, 2, 4, 8, 16, 32],
                    help="lanes per target of the main run's FP64 pair passes (SPH_OPT_LANES)")
    return ap.parse_args()


def make_case(name: str, dx: float | None):
    from mysph_gb300 import cases
    kw = {} if dx is None else {"dx": dx}
    return getattr(cases, name)(**kw)


def bench_config(case, precision: str) -> dict:
    """The `config` object of both arms (ours and --impl reference): the same
    keys and values for the same workload."""
    return {"workload": workload_name(case), "n_real": case.n_real, "n_wall": case.n_wall,
            "dim": case.dim, "precision": precision, "dt": case.params.dt,
            "l2": (f"inputs larger than L2 (129 MB): {case.n} particles, over "
                   f"{case.n * 200 / 1e6:.0f} MB of FP64 state fields" if case.n * 200 > 129e6 else
                   f"state of {case.n} particles fits in L2; no flush between steps")}


def workload_name(case) -> str:
    m = case.meta
    if case.name == "dam_break_3d":
        return (f"3-D dam break, block {m['block'][0]}x{m['block'][1]}x{m['block'][2]} m in "
                f"{m['box'][0]}x{m['box'][1]}x{m['box'][2]} m box, dx={m['dx']} m, "
                f"{case.n_real} fluid + {case.n_wall} wall particles")
    return f"{case.name} dx={m.get('dx')} ({case.n_real} real + {case.n_wall} wall particles)"


def dist_setup():
    from mysph_gb300.replicas import world
    return world()


class Clocks:
    """nvidia-smi samples during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
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
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(stage: str, config: str) -> tuple[float | None, float | None, int | None]:
    """Per-launch DRAM bytes and FP64 flops of a kernel from the committed ncu
    summary (profiles/<kernel>_<config>.md), scaled to the bench workload."""
    f = ROOT / "profiles" / f"{stage}_{config}.md"
    if not f.exists():
        return None, None, None
    txt = f.read_text()
    def grab(key):
        m = re.search(rf"^{key}:\s*([0-9.eE+-]+)", txt, re.M)
        return float(m.group(1)) if m else None
    return grab("dram_bytes_per_particle"), grab("fp64_flops_per_particle"), None


def _rss_gb() -> float:
    """Resident set of this process in GB (Linux /proc)."""
    try:
        for line in Path("/proc/self/status").read_text().splitlines():
            if line.startswith("VmRSS:"):
                return int(line.split()[1]) * 1024 / 1e9
    except (OSError, ValueError):
        pass
    return float("nan")


def _time_oracle(case, steps: int, warm: int, threads: int = 0, ram: dict | None = None):
    from oracle.oracle import Oracle
    t0 = time.perf_counter()
    rss0 = _rss_gb()
    o = Oracle(case, omp=True, threads=threads)
    setup = time.perf_counter() - t0
    if warm:
        o.advance(warm)
    t0 = time.perf_counter()
    o.advance(steps)
    dt = time.perf_counter() - t0
    cores = o.threads
    if ram is not None:
        ram["oracle_host_ram_gb"] = _rss_gb() - rss0
    del o
    return case.n_real * steps / dt, dt, setup, cores


def cpu_baseline(case, steps: int, warm: int = 1, config: str = "", dx: float | None = None) -> dict:
    ram = {}
    value, dt, setup, cores = _time_oracle(case, steps, warm, ram=ram)
    out = {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
           "sample": f"{steps} leap-frog steps of the full workload after {warm} warm-up step(s) "
                     f"(OpenMP oracle, {dt:.1f} s; setup {setup:.1f} s)",
           "seconds": dt, "host": host_cpu(), "omp_threads": "all host cores",
           "host_ram_gb": ram.get("oracle_host_ram_gb"),
           "host_ram_note": "resident-set growth of the process while the oracle holds the workload "
                            "(particles plus stored neighbour lists)"}
    # one thread, on the same geometry at twice the spacing (1/8 of the
    # particles in 3-D) so that the sample stays a few seconds
    try:
        small = make_case(config, (dx or case.meta.get("dx", 0.004)) * 2) if config else case
        v1, dt1, _, _ = _time_oracle(small, 1, 1, threads=1)
        out["single_thread"] = {"value": v1, "unit": METRIC, "cores": 1,
                                "sample": f"1 step of the same geometry at dx x2 ({small.n_real} real "
                                          f"particles), {dt1:.1f} s"}
    except Exception as ex:
        out["single_thread"] = {"value": None, "error": str(ex)[:200]}
    return out


def host_cpu() -> str:
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part")):
                return f"{os.cpu_count()} cores, {line.split(':', 1)[1].strip()}"
    except OSError:
        pass
    return f"{os.cpu_count()} cores"


def run_batched() -> dict:
    """256 independent 2-D dam breaks in one batch (mixed precision), next to
    the same batch in FP64 and the plain FP64 path one system at a time."""
    from mysph_gb300 import ensemble
    t0 = time.perf_counter()
    r = ensemble.run(count=256, steps=20)
    r["wall_s"] = time.perf_counter() - t0
    return r


def run_serving(count: int, real_capacity: int = 1_500_000, wall_capacity: int = 500_000) -> dict:
    """Poisson stream (mean 50 requests/s) of 2-D dam breaks and cantilevers
    of 1k-500k particles and 500-5000 steps, continuously batched.  The
    budget (real and wall particle slots reserved per model) is smaller than
    the stream's peak demand, so admission waits for capacity: the queueing
    delay and the run time are reported apart."""
    from mysph_gb300 import params as P
    from mysph_gb300 import serve
    reqs = serve.poisson_requests(count, rate=50.0, seed=4)
    srv = serve.Server(precision=P.PREC_MIXED, real_capacity=real_capacity, wall_capacity=wall_capacity,
                       max_instances=64)
    try:
        st = srv.run(reqs, chunk=64)
    finally:
        srv.close()
    st["workload"] = (f"{count} Poisson requests (seed 4, mean 50/s): 2-D dam break or steel cantilever, "
                      f"1k-500k particles, 500-5000 steps; mixed precision; HBM budget "
                      f"{real_capacity / 1e6:g}M real + {wall_capacity / 1e6:g}M wall particle slots per model "
                      f"({sum(st['hbm_reserved_bytes'].values()) / 1e9:.2f} GB reserved); each case generated "
                      f"on the device at admission (time-to-solution includes it); the two models' batches "
                      f"advance on their own streams")
    st["peak_demand_particles"] = _peak_demand(reqs)
    return st


def _peak_demand(reqs) -> int:
    """Real particles the stream would hold at once with no budget (each
    request resident from arrival for its measured run time)."""
    ev = sorted([(r.arrival, r.case.n_real) for r in reqs] +
                [(r.arrival + (r.done - r.admitted), -r.case.n_real) for r in reqs])
    cur = best = 0
    for _, d in ev:
        cur += d
        best = max(best, cur)
    return int(best)


def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    case = make_case(args.config, args.dx)
    from oracle.oracle import Oracle
    o = Oracle(case, omp=True)
    if args.warmup:
        o.advance(args.warmup)
    t0 = time.perf_counter()
    o.advance(args.steps)
    dt = time.perf_counter() - t0
    value = case.n_real * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(case, "fp64"),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": o.threads, "kind": "port",
                         "sample": f"{args.steps} leap-frog steps of the full workload after "
                                   f"{args.warmup} warm-up steps (C++/OpenMP restatement of the "
                                   f"reference; the Fortran reference cannot be built here)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_mixed(case, args, ref_fields, precision=None) -> dict:
    """Time the mixed-precision (or DF64) form on the same workload and
    compare its state after warm-up + timed steps with the FP64 run's."""
    import torch
    from mysph_gb300 import params as P
    from mysph_gb300.solver import GpuSolver
    prm = case.params.copy()
    prm.precision = P.PREC_MIXED if precision is None else precision
    s = GpuSolver(case, params=prm)
    s.advance(max(args.warmup, 3))
    stream = torch.cuda.ExternalStream(s.stream())
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.advance(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    err = {k: float(np.linalg.norm(s.field(k)[: case.n_real] - v) / np.linalg.norm(v))
           for k, v in ref_fields.items()}
    # per-stage times from further steps with a CUDA event around each stage
    # (the timed steps above replay the captured graph, without them)
    s.enable_stage_timing(True)
    s.advance(args.steps)
    stage_ms, nst = s.stage_times()
    s.close()
    per = {k: v / max(nst, 1) for k, v in stage_ms.items()}
    roof = None
    if prm.precision == P.PREC_MIXED and case.dim == 3 and per:
        dom = max(per, key=per.get)
        peak, kind = measured_peaks()
        algo = ALGO_BYTES_MIXED_3D[dom] * case.n_real
        ach = algo / (per[dom] / 1e3) / 1e9 if per[dom] > 0 else None
        bpp, _, _ = profile_traffic(dom + "_mixed", "dam_break_3d")
        roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak if ach else None, "algo_bytes_per_launch": algo,
                "traffic": bpp * case.n_real if bpp is not None else None,
                "peak_source": f"{kind} (MEASURED_PEAKS.json hbm_gbs)", "ms_per_launch": per[dom],
                "whole_step_frac": (472 * case.n_real * args.steps / (ms / 1e3) / 1e9) / peak}
    label = ("FP32 pair loops (Kahan sums), FP64 positions/integration" if prm.precision == P.PREC_MIXED
             else "double-float pair loops on the FP32 pipes (about 48 bits), FP64 neighbour test, "
                  "epilogues and integration")
    return {"value": case.n_real * args.steps / (ms / 1e3), "unit": METRIC, "ms_per_step": ms / args.steps,
            "precision": label, "roofline": roof,
            "stages_ms_per_step": per,
            "rel_l2_vs_fp64": err, "steps_compared": max(args.warmup, 3) + args.steps}


def run_long(case, steps: int) -> dict:
    """Advance the same workload `steps` steps in FP64, in mixed precision
    and in DF64 from one initial state, and state each field's error against
    the FP64 run (relative L2 over the real particles)."""
    from mysph_gb300 import params as P
    from mysph_gb300.solver import GpuSolver
    keys = ("RHO", "V", "X", "P")
    out = {}
    ref = None
    from mysph_gb300._lib import SphError
    for name, prec in (("fp64", P.PREC_FP64), ("mixed", P.PREC_MIXED), ("df64", P.PREC_DF64)):
        prm = case.params.copy()
        prm.precision = prec
        try:
            s = GpuSolver(case, params=prm)
        except SphError as ex:   # DF64 covers fluid systems only
            out[name] = f"unsupported: {ex}"
            continue
        with s:
            e0 = s.energy()
            ms = _timed_advance(s, steps)
            f = {k: s.field(k)[: case.n_real] for k in keys}
            t = s.info()["time"]
            en = s.energy()
        rate = {"value": case.n_real * steps / (ms / 1e3), "unit": METRIC, "ms_per_step": ms / steps,
                "energy_start": e0, "energy_end": en}
        if ref is None:
            ref = f
            ref_e = en
            out["time"] = t
            out[name] = rate
            continue
        out[name] = dict(rate, rel_l2_vs_fp64={
            k: float(np.linalg.norm(f[k] - ref[k]) / np.linalg.norm(ref[k])) for k in keys},
            energy_rel_vs_fp64={k: abs(en[k] - ref_e[k]) / abs(ref_e[k]) for k in ("kinetic", "total")})
    out["steps"] = steps
    return out


def _timed_advance(solver, steps: int) -> float:
    """ms of `steps` steps on the solver's stream (CUDA events)."""
    import torch
    stream = torch.cuda.ExternalStream(solver.stream())
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.advance(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


CFG0_LANES = (1, 2, 4, 8, 16)


def run_cfg0(steps: int = 1000, oracle: bool = True) -> dict:
    """The 2-D dam break of 5,000 fluid particles (dx = 2 cm, 1.0 x 2.0 m
    column in a 4.0 x 3.0 m tank), plain FP64, over its 1,000 steps from
    rest: the GPU's time for the whole run (first step and graph capture
    included), its pass-B roofline, the OpenMP oracle's time for the same
    run on the host cores, and the GPU state against the oracle's at t_end."""
    from mysph_gb300 import cases
    from mysph_gb300 import params as P
    from mysph_gb300.solver import GpuSolver
    case = cases.dam_break_2d()
    nr = case.n_real

    def one_run(lanes):
        with GpuSolver(case) as w:  # warm the library (module load, first launches)
            w.set_option(P.OPT_LANES, lanes)
            w.advance(3)
        with GpuSolver(case) as s:
            s.set_option(P.OPT_LANES, lanes)
            ms = _timed_advance(s, steps)
            got = {k: s.field(k)[:nr] for k in ("RHO", "V", "X", "P")}
            t_end = s.info()["time"]
            s.enable_stage_timing(True)
            s.advance(50)   # per-stage times (eager launches with an event around each stage)
            stage_ms, nst = s.stage_times()
        return ms, got, t_end, {k: v / max(nst, 1) for k, v in stage_ms.items()}

    runs = {lanes: one_run(lanes) for lanes in CFG0_LANES}
    best = min(runs, key=lambda k: runs[k][0])
    ms, got, t_end, per = runs[best]
    peak, kind = measured_peaks()
    algo = ALGO_BYTES[2]["pass_b"] * nr
    ach = algo / (per["pass_b"] / 1e3) / 1e9 if per.get("pass_b") else None
    out = {"workload": workload_name(case) + f", plain FP64, {steps} steps from rest",
           "value": nr * steps / (ms / 1e3), "unit": METRIC, "ms_per_step": ms / steps, "lanes": best,
           "stages_ms_per_step": per, "stages_note": "50 further steps, each stage bracketed by CUDA events "
                                                       "(eager launches; the timed run replays a CUDA graph)",
           "time_s": t_end,
           "roofline_pass_b": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                               "frac": ach / peak if ach else None, "algo_bytes_per_launch": algo,
                               "note": "5,000 targets per launch: the kernel is launch- and latency-bound"},
           "by_lanes": {str(k): {"value": nr * steps / (r[0] / 1e3), "ms_per_step": r[0] / steps,
                                 "pass_a_ms": r[3].get("pass_a"), "pass_b_ms": r[3].get("pass_b")}
                        for k, r in runs.items()},
           "lanes_note": "SPH_OPT_LANES: lanes per target of the FP64 passes A and B; `value` is the "
                         "fastest, `by_lanes` every setting timed (1 is the default)"}
    if oracle:
        from oracle.oracle import Oracle
        o = Oracle(case, omp=True)
        t0 = time.perf_counter()
        o.advance(steps)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": nr * steps / dt, "unit": METRIC, "cores": o.threads, "kind": "port",
                               "sample": f"the same {steps} steps (OpenMP oracle, {dt:.1f} s)"}
        rel = lambda g: {k: float(np.linalg.norm(g[k] - o.field(k)[:nr]) / np.linalg.norm(o.field(k)[:nr]))
                         for k in g}
        out["rel_l2_vs_oracle_at_t_end"] = rel(got)
        for k, r in runs.items():
            out["by_lanes"][str(k)]["rel_l2_vs_oracle_at_t_end"] = rel(r[1])
    return out


def run_cfg2(steps: int) -> dict:
    """The elastic gate at dx = 0.5 mm (322,000 real particles): FP64 and
    mixed precision from one initial state over a window of `steps` steps,
    each timed, with the mixed fields' error against FP64 at the end of the
    window and the largest speed (the gate stays bounded in this window; it
    grows without bound later, in the oracle as on the GPU)."""
    from mysph_gb300 import cases
    from mysph_gb300 import params as P
    from mysph_gb300.solver import GpuSolver
    case = cases.gate_2d()
    nr = case.n_real
    out = {"workload": workload_name(case) + f"; window of {steps} steps", "unit": METRIC}
    ref = None
    for name, prec in (("fp64", P.PREC_FP64), ("mixed", P.PREC_MIXED)):
        prm = case.params.copy()
        prm.precision = prec
        with GpuSolver(case, params=prm) as s:
            s.advance(3)
            ms = _timed_advance(s, steps - 3)
            f = {k: s.field(k)[:nr] for k in ("RHO", "V", "X", "P", "SHEAR")}
            out[name] = {"value": nr * (steps - 3) / (ms / 1e3), "ms_per_step": ms / (steps - 3),
                         "max_speed": float(np.linalg.norm(f["V"], axis=1).max()),
                         "time_s": s.info()["time"]}
        if ref is None:
            ref = f
        else:
            out[name]["rel_l2_vs_fp64"] = {k: float(np.linalg.norm(f[k] - ref[k]) / np.linalg.norm(ref[k]))
                                           for k in f}
    out["steps"] = steps
    return out


def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from mysph_gb300.solver import GpuSolver, probe_fp64_gflops

    case = make_case(args.config, args.dx)
    dim = case.dim
    fp64_peak = probe_fp64_gflops()
    main_prm = case.params.copy()
    if args.precision != "fp64":
        from mysph_gb300 import params as P
        main_prm.precision = P.PREC_MIXED if args.precision == "mixed" else P.PREC_DF64
        args.no_mixed = True
    solver = GpuSolver(case, params=main_prm)
    if args.lanes != 1:
        from mysph_gb300 import params as P
        solver.set_option(P.OPT_LANES, args.lanes)
    solver.advance(max(args.warmup, 3))
    stream = torch.cuda.ExternalStream(solver.stream())
    launches0 = solver.launch_count()
    clocks = Clocks(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    maxc, meanc = solver.advance(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1)
    launches = solver.launch_count() - launches0
    # the state the other precisions compare against: after warm-up + timed steps
    ref_fields = {k: solver.field(k)[: case.n_real] for k in ("RHO", "V", "X", "P")}
    # per-stage times from further steps with a CUDA event around each stage
    # (the timed steps above replay the captured two-step graph, without them)
    solver.enable_stage_timing(True)
    solver.advance(args.steps)
    stage_ms, nst = solver.stage_times()
    solver.enable_stage_timing(False)
    from mysph_gb300.replicas import max_over_ranks
    ms = max_over_ranks(ms, device="cuda")   # the job's time is its slowest replica
    value = case.n_real * args.steps * world / (ms / 1e3)

    # roofline of the dominant kernel
    per_launch = {k: v / max(nst, 1) for k, v in stage_ms.items()}
    dom = max(per_launch, key=per_launch.get)
    algo = ALGO_BYTES[dim][dom] * case.n_real
    peak, peak_kind = measured_peaks()
    achieved = algo / (per_launch[dom] / 1e3) / 1e9 if per_launch[dom] > 0 else None
    bpp, fpp, _ = profile_traffic(dom, args.config)
    traffic = bpp * case.n_real if bpp is not None else None
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": traffic,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s", "algo_bytes_per_launch": algo,
            "ms_per_launch": per_launch[dom]}
    if args.precision == "fp64":
        roof["note"] = "the FP64 pair passes are bound by FP64 issue, not by HBM: roofline_fp64 is the binding roof"
    roof64 = None
    if fpp is not None:
        ach = fpp * case.n_real / (per_launch[dom] / 1e3) / 1e9
        roof64 = {"bound": "fp64", "kernel": dom, "achieved": ach, "peak": fp64_peak, "unit": "GFLOP/s",
                  "frac": ach / fp64_peak, "peak_source": "measured FMA-chain probe (sph_probe_fp64_gflops)"}

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        nr = case.n_real
        pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True)
        hx, hv, hr, he = pin(nr * dim), pin(nr * dim), pin(nr), pin(nr)
        full_x, full_v = solver.field("X"), solver.field("V")
        hx.numpy()[:] = full_x[:nr].ravel()
        hv.numpy()[:] = full_v[:nr].ravel()
        hr.numpy()[:] = solver.field("RHO")[:nr]
        he.numpy()[:] = solver.field("E")[:nr]
        ptr = lambda t: __import__("ctypes").cast(t.data_ptr(), __import__("ctypes").POINTER(__import__("ctypes").c_double))
        for _ in range(2):
            solver._call("sph_step_host", 1, ptr(hx), ptr(hv), ptr(hr), ptr(he), None)
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            solver._call("sph_step_host", 1, ptr(hx), ptr(hv), ptr(hr), ptr(he), None)
        te = time.perf_counter() - t0
        te = max_over_ranks(te, device="cuda")
        b = nr * (2 * dim + 2) * 8
        e2e = {"value": nr * args.steps * world / te, "unit": METRIC, "h2d_bytes_per_step": b,
               "d2h_bytes_per_step": b, "ms_per_step": te * 1e3 / args.steps,
               "call": "sph_step_host(ctx, 1, x, v, rho, e, NULL) per step, pinned host buffers"}

    # the same workload with FP32 pair loops (SPH_PREC_MIXED), from the same
    # initial state over the same steps; per-field relative L2 against FP64
    mixed = df64 = None
    if not args.no_mixed:
        from mysph_gb300 import params as P
        mixed = run_mixed(case, args, ref_fields)
        df64 = run_mixed(case, args, ref_fields, P.PREC_DF64)
    long_run = None
    if args.long_run > 0 and rank == 0 and args.config == "dam_break_3d":
        long_run = run_long(case, args.long_run)
    cfg0 = cfg2 = None
    if rank == 0 and world == 1 and not args.no_configs:
        cfg0 = run_cfg0(oracle=not args.no_cpu)
        cfg2 = run_cfg2(args.gate_window)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(case, args.cpu_steps, config=args.config, dx=args.dx)
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "unit": METRIC, "error": str(ex)[:200]}

    # neighbour pairs per step at the end of the run (interactions/s)
    solver.nnps()
    pairs = int(solver.neighbor_counts().astype(np.int64).sum())
    dev_bytes = solver.device_bytes()
    solver.close()
    batched = serving = None
    if rank == 0 and world == 1:
        if not args.no_batched:
            batched = run_batched()
        if not args.no_serving:
            serving = run_serving(args.serve_requests)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (deterministic lattice of the named geometry)",
        "config": bench_config(case, args.precision),
        "parallelism": f"replicas x{world}", "lanes_per_target": args.lanes, "device_state_gb": dev_bytes / 1e9,
        "roofline": roof, "roofline_fp64": roof64, "fp64_peak_gflops": fp64_peak,
        "mixed": mixed, "df64": df64, "cfg1_long": long_run, "cfg0": cfg0, "cfg2": cfg2,
        "cpu_baseline": cpu, "e2e": e2e,
        "clocks": clk, "gpu_launches": launches,
        "stages_ms_per_step": per_launch, "courant": {"max": maxc, "mean": meanc},
        "pair_interactions_per_s": pairs * args.steps * world / (ms / 1e3),
        "pairs_per_step": pairs,
        "batched": batched, "serving": serving,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
