"""Batched ensemble of 2-D dam breaks, and the autotuner of its launch tiles.

The ensemble is a seeded set of independent dam-break columns (aspect ratio
in [0.25, 2], particle count log-uniform in [2k, 60k], dx in [5, 20] mm),
each with its own time step from its own CFL condition.  All of them live in
one batch context: every stage of a step is one launch over all systems, and
steady-state steps replay as a captured CUDA graph.

The autotuner times a few steps of the actual batch and descends one knob at
a time: cell size (factor x 2h, a new batch per value), then threads per
block and neighbour-list length of the mixed pair passes and the shared-
memory carveout (context options on the same batch).  The best setting per
(dim, size bucket, system count, precision) goes to a JSON cache.
"""
from __future__ import annotations

import json
import math
import os
import time
from pathlib import Path

import numpy as np

from . import cases
from . import params as P
from .solver import GpuBatch, GpuSolver

CACHE = Path(os.environ.get("MYSPH_TUNE_CACHE", Path(__file__).resolve().parent / "_build" / "autotune.json"))

# the autotuner's knobs: cell size (x 2h), threads per block and list length
# of the mixed pair passes, shared-memory carveout of the pair passes
SPACE = {
    "cell_factor": (1.0, 1.15, 1.3),
    "block": (32, 64, 128),
    "list_len": (64, 88, 120),
    "carveout": (-1, 100),
    "persistent": (0, 1),
}


def tune_key(dim: int, n_real: int, precision: int, n_inst: int) -> str:
    return f"dim{dim}-n2^{int(math.log2(max(n_real, 1)))}-inst2^{int(math.log2(max(n_inst, 1)))}-prec{precision}"


def _load_cache() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except Exception:
        return {}


def _save_cache(c: dict) -> None:
    try:
        CACHE.parent.mkdir(parents=True, exist_ok=True)
        CACHE.write_text(json.dumps(c, indent=1, sort_keys=True))
    except OSError:
        pass


def member_params(case, precision: int, cell_factor: float) -> P.SphParams:
    prm = case.params.copy()
    prm.precision = precision
    prm.cell_size = cell_factor * 2.0 * float(case.h.max()) * (1.0 + 1e-9)
    return prm


def build_batch(members, precision: int, cell_factor: float = 1.0, spare: float = 0.0) -> GpuBatch:
    nr = sum(m.n_real for m in members)
    nw = sum(m.n_wall for m in members)
    base = members[0].params.copy()
    base.precision = precision
    b = GpuBatch(base, len(members), int(nr * (1 + spare)) + 1, int(nw * (1 + spare)) + 1)
    b.member_ids = [b.add(m, params=member_params(m, precision, cell_factor)) for m in members]
    return b


def time_steps(obj, steps: int) -> float:
    """Milliseconds of `steps` steps, CUDA events on the object's stream."""
    import torch
    stream = torch.cuda.ExternalStream(obj.stream())
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    obj.advance(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def apply_options(b, cfg: dict) -> None:
    b.set_option(P.OPT_SMEM_CARVEOUT, cfg["carveout"])
    b.set_option(P.OPT_BLOCK_SIZE, cfg["block"])
    b.set_option(P.OPT_LIST_LEN, cfg["list_len"])
    b.set_option(P.OPT_PERSISTENT, cfg.get("persistent", 0))


def autotune(members, precision: int, steps: int = 6, use_cache: bool = True) -> dict:
    dim = members[0].dim
    n = sum(m.n_real for m in members)
    key = tune_key(dim, n, precision, len(members))
    cache = _load_cache()
    if use_cache and key in cache:
        return dict(cache[key], cached=True)
    best = {"cell_factor": 1.0, "block": 128, "list_len": 64 if dim == 2 else 88, "carveout": -1, "persistent": 0}
    trials = []

    def timed(b, cfg):
        apply_options(b, cfg)
        b.advance(4)
        ms = time_steps(b, steps) / steps
        trials.append(dict(cfg, ms_per_step=ms))
        return ms

    # cell size: one batch per value
    best_ms, best_b = None, None
    for f in SPACE["cell_factor"]:
        cfg = dict(best, cell_factor=f)
        b = build_batch(members, precision, f)
        ms = timed(b, cfg)
        if best_ms is None or ms < best_ms:
            if best_b is not None:
                best_b.close()
            best, best_ms, best_b = cfg, ms, b
        else:
            b.close()
    # the launch knobs, one at a time, on the batch of the best cell size
    try:
        for knob in ("block", "list_len", "carveout", "persistent"):
            for v in SPACE[knob]:
                if v == best[knob]:
                    continue
                cfg = dict(best, **{knob: v})
                ms = timed(best_b, cfg)
                if ms < best_ms:
                    best, best_ms = cfg, ms
    finally:
        best_b.close()
    result = dict(best=dict(best, ms_per_step=best_ms), trials=trials, key=key)
    cache[key] = result
    _save_cache(cache)
    return dict(result, cached=False)


def _rel_l2(b, b64, ids, fields) -> dict:
    """Relative L2 of the batched fields against the FP64 batch over every
    member's real particles."""
    out = {}
    for f in fields:
        num = den = 0.0
        for k, (nr, _) in ids:
            a = b.field(k, f)[:nr]
            r = b64.field(k, f)[:nr]
            num += float(np.sum((a - r) ** 2))
            den += float(np.sum(r ** 2))
        out[f] = math.sqrt(num / den) if den > 0 else 0.0
    return out


def _to_time(b, ids, n_steps: dict, fields) -> dict:
    """Advance a batch until each member has taken its own n_steps[k] steps
    (members leave the batch when they reach their count: continuous
    batching), and return each member's fields at that point."""
    out = {}
    done = 0
    for n in sorted(set(n_steps.values())):
        if n > done:
            b.advance(n - done)
            done = n
        for k, (nr, _) in ids:
            if n_steps[k] == n:
                out[k] = {f: b.field(k, f)[:nr] for f in fields}
                b.remove(k)
    return out


def run(count: int = 256, seed: int = 20261203, steps: int = 20, warmup: int = 3,
        precision: int = P.PREC_MIXED, plain_sample: int = 16, tune: bool = True,
        t_end_s: float = 0.01) -> dict:
    """Batched throughput of the ensemble, next to the same batch in FP64 and
    the plain FP64 path (one system at a time, timed on a sample of the same
    members), and the two launch forms of the pair passes (one block per tile
    of targets, or a persistent grid).  Then fresh batches in both
    precisions run every member to the physical time t_end_s (each member
    its own number of steps of its own dt, leaving the batch when done) and
    the batched fields are compared with the FP64 ones there."""
    specs = cases.ensemble_specs(count=count, seed=seed)
    members = [cases.ensemble_member(s) for s in specs]
    n_real = sum(m.n_real for m in members)
    default = {"cell_factor": 1.0, "block": 128, "list_len": 64, "carveout": -1, "persistent": 0}
    tuned = autotune(members, precision) if tune else dict(best=default)
    cfg = dict(default, **tuned["best"])
    warm = max(warmup, 3)
    b = build_batch(members, precision, cfg["cell_factor"])
    try:
        apply_options(b, cfg)
        b.advance(warm)
        launches0 = b.launch_count()
        ms = time_steps(b, steps)
        launches = b.launch_count() - launches0
        # the other launch form of the pair passes on the same batch
        other = dict(cfg, persistent=1 - int(cfg.get("persistent", 0)))
        apply_options(b, other)
        b.advance(2)
        ms_other = time_steps(b, steps)
        forms = {("persistent" if cfg.get("persistent") else "per_tile"): ms / steps,
                 ("persistent" if other["persistent"] else "per_tile"): ms_other / steps}
    finally:
        b.close()
    # the same batch in FP64 (batching without the precision change)
    b64 = build_batch(members, P.PREC_FP64, cfg["cell_factor"])
    try:
        b64.set_option(P.OPT_SMEM_CARVEOUT, cfg["carveout"])
        b64.advance(warm)
        ms64 = time_steps(b64, steps)
    finally:
        b64.close()
    # every member to the physical time t_end_s, in both precisions
    n_steps = {}
    fields = ("RHO", "V", "X", "P")
    res = {}
    for prec in (precision, P.PREC_FP64):
        bb = build_batch(members, prec, cfg["cell_factor"])
        try:
            if prec == precision:
                apply_options(bb, cfg)
            ids = sorted(bb.sizes.items())
            if not n_steps:
                n_steps = {k: max(int(math.ceil(t_end_s / m.params.dt - 1e-9)), 1)
                           for k, m in zip(bb.member_ids, members)}
            res[prec] = _to_time(bb, ids, n_steps, fields)
        finally:
            bb.close()
    err = {}
    for f in fields:
        num = sum(float(np.sum((res[precision][k][f] - res[P.PREC_FP64][k][f]) ** 2)) for k in n_steps)
        den = sum(float(np.sum(res[P.PREC_FP64][k][f] ** 2)) for k in n_steps)
        err[f] = math.sqrt(num / den) if den > 0 else 0.0
    # plain FP64, one system at a time, on an evenly spaced sample
    idx = np.linspace(0, count - 1, min(plain_sample, count)).round().astype(int)
    ps, tsum = 0, 0.0
    for i in idx:
        m = members[i]
        with GpuSolver(m) as s:
            s.advance(warm)
            tsum += time_steps(s, steps) / 1e3
            ps += m.n_real * steps
    plain = ps / tsum
    batched = n_real * steps / (ms / 1e3)
    batched64 = n_real * steps / (ms64 / 1e3)
    return {
        "workload": f"{count} independent 2-D dam breaks (seed {seed}), {n_real} real particles in total",
        "n_instances": count, "n_real": n_real,
        "n_wall": sum(m.n_wall for m in members),
        "value": batched, "unit": "particle-steps/s", "ms_per_step": ms / steps,
        "precision": "FP32 pair loops, FP64 positions/integration" if precision == P.PREC_MIXED else "fp64",
        "batched_fp64": batched64,
        "plain_fp64_one_at_a_time": plain, "plain_sample": int(len(idx)),
        "speedup_vs_plain_fp64": batched / plain,
        "speedup_vs_batched_fp64": batched / batched64,
        "gpu_launches_per_step": launches / steps,
        "launch_forms_ms_per_step": forms,
        "rel_l2_vs_fp64_at_t_end": err, "t_end_s": t_end_s,
        "t_end_steps_range": [min(n_steps.values()), max(n_steps.values())],
        "autotune": {"best": cfg, "cached": tuned.get("cached", False),
                     "trials": tuned.get("trials")},
    }
