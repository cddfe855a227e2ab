"""Serving: a device-resident request loop with continuous batching.

Requests (a 2-D dam break or a 2-D steel cantilever, each with its own size
and step count) arrive at seeded Poisson times; each is described by a few
lattice blocks that the device expands at admission.  The server keeps one batch
context per model (fluid, solid); each batch reserves its device memory up
front, which is the HBM budget: a request is admitted as soon as its batch
has free particle and instance slots, and its state stays on the device
until its last step.  Every loop iteration queues, on each busy batch's own
stream, the steps up to that batch's next completion, then waits for both,
so the two models' device work overlaps; requests that arrive while others
run join them in the same launches; finished requests are read back and
their slots freed.  Time-to-solution = completion time - arrival time; it
is the queueing delay (admission - arrival, while the budget is full) plus
the run time (completion - admission).
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import cases
from . import params as P
from .solver import GpuBatch


@dataclass
class Request:
    rid: int
    kind: str            # "dam_break" or "cantilever"
    n_target: int
    steps: int
    arrival: float       # seconds after the start
    seed: int
    case: object = None
    # filled by the server
    inst: int = -1
    admitted: float = -1.0
    done: float = -1.0
    result: dict = field(default_factory=dict)


def make_case(kind: str, n_target: int, seed: int, precision: int, on_device: bool = True):
    """A request's system: a dam-break column of about n_target particles with
    a seeded aspect ratio, or a 10:1 steel cantilever of about n_target.  By
    default a block description the device expands (cases.BlockCase); with
    on_device=False the same particles as host arrays (cases.Case)."""
    rng = np.random.default_rng(seed)
    if kind == "dam_break":
        aspect = rng.uniform(0.5, 2.0)
        dx = 0.01
        w = dx * math.sqrt(n_target / aspect)
        gen = cases.dam_break_2d_blocks if on_device else cases.dam_break_2d
        c = gen(dx=dx, width=max(round(w / dx), 4) * dx, height=max(round(aspect * w / dx), 4) * dx,
                tank_w=4.0 * w + 8 * dx, tank_h=1.5 * aspect * w + 4 * dx)
    else:
        dx = 1e-3
        t_cells = max(int(round(math.sqrt(n_target / 10.0))), 3)
        gen = cases.cantilever_2d_blocks if on_device else cases.cantilever_2d
        c = gen(dx=dx, length=10 * t_cells * dx, thickness=t_cells * dx)
    c.params = c.params.copy()
    c.params.precision = precision
    return c


def poisson_requests(count: int, rate: float, seed: int, n_lo: int = 1000, n_hi: int = 500_000,
                     s_lo: int = 500, s_hi: int = 5000, kinds=("dam_break", "cantilever")) -> list[Request]:
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        n = int(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi))))
        out.append(Request(rid, kinds[int(rng.integers(len(kinds)))], n, int(rng.integers(s_lo, s_hi + 1)),
                           t, int(rng.integers(1 << 30))))
    return out


class Server:
    """One batch per model; admission by the batches' reserved capacity."""

    def __init__(self, precision: int = P.PREC_MIXED, real_capacity: int = 4_000_000,
                 wall_capacity: int = 1_000_000, max_instances: int = 64):
        self.precision = precision
        proto = {"dam_break": make_case("dam_break", 2000, 0, precision),
                 "cantilever": make_case("cantilever", 2000, 0, precision)}
        self.batches = {k: GpuBatch(c.params, max_instances, real_capacity,
                                    wall_capacity if k == "dam_break" else 1)
                        for k, c in proto.items()}

    def close(self):
        for b in self.batches.values():
            b.close()

    def _fits(self, b: GpuBatch, c) -> bool:
        cap = b.capacity()
        return cap["free_slots"] > 0 and cap["free_real"] >= c.n_real and cap["free_wall"] >= c.n_wall

    def run(self, requests: list[Request], keep_fields=("X", "V", "RHO"), chunk: int = 64,
            clock=time.perf_counter) -> dict:
        """Serve the requests; a request's case is built when it arrives (a
        block description, expanded on the device at admission), so its
        time-to-solution includes the case set-up."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        active: dict[str, dict[int, Request]] = {k: {} for k in self.batches}
        remaining: dict[int, int] = {}
        t0 = clock()
        busy_steps = 0
        while pending or any(active.values()):
            now = clock() - t0
            # admission: arrived requests in arrival order, while they fit
            waiting = deque()
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                if r.case is None:
                    r.case = make_case(r.kind, r.n_target, r.seed, self.precision)
                b = self.batches[r.kind]
                if self._fits(b, r.case):
                    r.inst = b.add_blocks(r.case) if isinstance(r.case, cases.BlockCase) else b.add(r.case)
                    r.admitted = clock() - t0
                    active[r.kind][r.inst] = r
                    remaining[r.rid] = r.steps
                else:
                    waiting.append(r)
            pending.extendleft(reversed(waiting))
            if not any(active.values()):
                if pending:
                    wait = pending[0].arrival - (clock() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                continue
            # advance every busy batch up to its next completion (even chunks
            # keep the captured step graph reusable).  The batches' steps are
            # queued on their own streams back to back and waited for
            # afterwards, so the models' device work overlaps.
            step_of = {}
            for kind, b in self.batches.items():
                if not active[kind]:
                    continue
                k = min(chunk, min(remaining[r.rid] for r in active[kind].values()))
                b.advance_async(k)
                step_of[kind] = k
            for kind, k in step_of.items():
                b = self.batches[kind]
                b.sync()
                busy_steps += k
                for r in list(active[kind].values()):
                    remaining[r.rid] -= k
                    if remaining[r.rid] == 0:
                        r.result = {f: b.field(r.inst, f)[: r.case.n_real] for f in keep_fields}
                        r.done = clock() - t0
                        b.remove(r.inst)
                        del active[kind][r.inst]
        makespan = clock() - t0
        tts = np.array([r.done - r.arrival for r in requests])
        queue = np.array([r.admitted - r.arrival for r in requests])
        run = np.array([r.done - r.admitted for r in requests])
        work = sum(r.case.n_real * r.steps for r in requests)
        pct = lambda a, q: float(np.percentile(a, q))
        return {
            "requests": len(requests),
            "p50_tts_s": pct(tts, 50),
            "p99_tts_s": pct(tts, 99),
            "mean_tts_s": float(tts.mean()),
            "p50_queue_s": pct(queue, 50),
            "p99_queue_s": pct(queue, 99),
            "max_queue_s": float(queue.max()),
            "p50_run_s": pct(run, 50),
            "p99_run_s": pct(run, 99),
            "waited": int(np.sum(queue > 0.05)),
            "max_concurrent": max_concurrency(requests),
            "makespan_s": makespan,
            "particle_steps": int(work),
            "value": work / makespan,
            "unit": "particle-steps/s",
            "hbm_reserved_bytes": {k: b.device_bytes() for k, b in self.batches.items()},
        }


def max_concurrency(requests: list[Request]) -> int:
    """Most requests resident on the device at one time."""
    ev = sorted([(r.admitted, 1) for r in requests] + [(r.done, -1) for r in requests],
                key=lambda e: (e[0], e[1]))
    cur = best = 0
    for _, d in ev:
        cur += d
        best = max(best, cur)
    return best
