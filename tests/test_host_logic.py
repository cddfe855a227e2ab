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


def _d2f_bits(b):
    """The bit algorithm of d2f (csrc/sph_device.cuh) on uint64 patterns,
    for results in the normal float range (the others take the conversion
    instruction there): sign, exponent rebased by 896, the top 23 fraction
    bits, plus one above half or at half with the kept fraction odd."""
    b = b.astype(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    e = ((hi >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64) - 896
    low = (b & np.uint64(0x1FFFFFFF)).astype(np.uint32)
    r = (hi & np.uint32(0x80000000)) | (np.clip(e, 0, 255).astype(np.uint32) << np.uint32(23)) | \
        ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)).astype(np.uint32)
    up = (low > 0x10000000) | ((low == 0x10000000) & ((r & np.uint32(1)) == 1))
    return (r + up.astype(np.uint32)).astype(np.uint32), (e >= 1) & (e <= 253)


def test_integer_double_to_float_rounding():
    """d2f's bit algorithm gives IEEE round-to-nearest-even (numpy's
    float64 -> float32) on every double in the normal float range: random
    fractions, exact ties and their neighbours, and mantissas that carry
    into the exponent."""
    rng = np.random.default_rng(7)
    n = 200_000
    e = rng.integers(897, 1150, n, dtype=np.uint64)
    frac = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    sign = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    base = sign | (e << np.uint64(52)) | frac
    tie = (base & ~np.uint64(0x1FFFFFFF)) | np.uint64(0x10000000)
    cases = [base, tie, tie + np.uint64(1), tie - np.uint64(1),
             sign | (e << np.uint64(52)) | np.uint64((1 << 52) - 1)]   # all ones: carries
    for b in cases:
        got, ok = _d2f_bits(b)
        want = b.view(np.float64).astype(np.float32).view(np.uint32)
        assert ok.all()
        assert np.array_equal(got, want)


def test_multiply_shift_cell_division():
    """The grid's multiply-shift reciprocals (grid_divisors in csrc/sph_ctx.cu,
    cell_from_key in csrc/sph_device.cuh): l = ceil(log2 nc), m = ceil(2^(31+l)
    / nc), and (n m) >> (31 + l) == n // nc for 0 <= n < 2^31, the range of
    the cell keys; m stays below 2^33, so n m fits 64 bits."""
    rng = np.random.default_rng(11)
    divisors = [1, 2, 3, 5, 7, 63, 64, 65, 84, 167, 4095, 4096, 4097, (1 << 24) - 1, 1 << 24]
    divisors += [int(v) for v in rng.integers(1, 1 << 24, 200)]
    for dv in divisors:
        l = 0
        while (1 << l) < dv:
            l += 1
        m = ((1 << (31 + l)) + dv - 1) // dv
        assert m < (1 << 33)
        ns = [0, 1, dv - 1, dv, dv + 1, (1 << 31) - 1, (1 << 31) - dv]
        ns += [int(v) for v in rng.integers(0, 1 << 31, 500)]
        for n in ns:
            assert (n * m) >> (31 + l) == n // dv, (n, dv)
