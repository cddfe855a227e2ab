"""Host logic of the ensemble and the server, on the CPU with fake batches.

The fakes stand in for a batch context: they count the steps each live
system has taken, report free capacity, and return a system's step count as
its field, so the tests check what the host loops do (how many steps each
system gets, when requests are admitted, what the statistics say) without a
GPU.
"""
import numpy as np

from mysph_gb300 import ensemble, serve
from mysph_gb300 import params as P


class FakeBatch:
    """The calls of GpuBatch that the host loops make."""

    def __init__(self, real_capacity=10**9, wall_capacity=10**9, slots=1024, clock=None):
        self.real_cap, self.wall_cap, self.slot_cap = real_capacity, wall_capacity, slots
        self.live = {}          # inst -> [steps, n_real, n_wall]
        self.next_id = 0
        self.queued = 0
        self.clock = clock
        self.sizes = {}

    def _add(self, nr, nw):
        k = self.next_id
        self.next_id += 1
        self.live[k] = [0, nr, nw]
        self.sizes[k] = (nr, nw)
        return k

    def add(self, case, params=None):
        return self._add(case.n_real, case.n_wall)

    def add_blocks(self, bc, params=None):
        return self._add(*bc.counts())

    def remove(self, k):
        del self.live[k]
        self.sizes.pop(k, None)

    def capacity(self):
        used_r = sum(v[1] for v in self.live.values())
        used_w = sum(v[2] for v in self.live.values())
        return dict(free_real=self.real_cap - used_r, free_wall=self.wall_cap - used_w,
                    free_slots=self.slot_cap - len(self.live))

    def advance(self, k):
        for v in self.live.values():
            v[0] += k
        if self.clock is not None:
            self.clock.t += 1e-4 * k

    def advance_async(self, k):
        self.queued += k

    def sync(self):
        k, self.queued = self.queued, 0
        self.advance(k)
        return 0.0, 0.0

    def field(self, k, name):
        steps, nr, nw = self.live[k]
        return np.full(nr + nw, float(steps))

    def device_bytes(self):
        return 1000

    def close(self):
        pass


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-6
        return self.t


def test_to_time_gives_each_member_its_own_steps():
    b = FakeBatch()
    for k in range(6):
        b._add(10 + k, 3)
    ids = sorted(b.sizes.items())
    n_steps = {k: s for (k, _), s in zip(ids, (74, 385, 74, 120, 300, 1))}
    out = ensemble._to_time(b, ids, n_steps, ("X",))
    assert set(out) == set(n_steps)
    for k, (nr, _) in ids:
        assert len(out[k]["X"]) == nr
        assert np.all(out[k]["X"] == n_steps[k])
    assert not b.live   # every member left the batch at its count


def _server(real_capacity, clock):
    srv = serve.Server.__new__(serve.Server)
    srv.precision = P.PREC_MIXED
    srv.batches = {k: FakeBatch(real_capacity=real_capacity, clock=clock) for k in ("dam_break", "cantilever")}
    return srv


def test_server_admits_within_budget_and_runs_each_request_its_steps():
    clock = FakeClock()
    reqs = serve.poisson_requests(30, rate=2000.0, seed=11, n_lo=1000, n_hi=20_000, s_lo=50, s_hi=400)
    srv = _server(40_000, clock)
    st = srv.run(reqs, keep_fields=("X",), chunk=32, clock=clock)
    assert st["requests"] == 30
    for r in reqs:
        # each request took exactly its own number of steps, and was read
        # back after its last one
        assert np.all(r.result["X"] == r.steps), (r.rid, r.steps, r.result["X"][:1])
        assert r.arrival <= r.admitted <= r.done
    # the budget binds: at no time do a model's resident requests exceed it
    for kind in ("dam_break", "cantilever"):
        ev = sorted([(r.admitted, r.case.n_real) for r in reqs if r.kind == kind] +
                    [(r.done, -r.case.n_real) for r in reqs if r.kind == kind], key=lambda e: (e[0], e[1]))
        cur = 0
        for _, d in ev:
            cur += d
            assert cur <= 40_000
    assert st["waited"] > 0 and st["max_concurrent"] < 30
    assert st["p99_queue_s"] >= st["p50_queue_s"] >= 0.0
    assert st["p99_tts_s"] >= st["p50_tts_s"] > 0.0
    assert st["particle_steps"] == sum(r.case.n_real * r.steps for r in reqs)
