"""Continuous batching: requests that arrive while others run join the same
launches, and each result equals the same case run alone (bit for bit: a
system's arithmetic does not depend on the other systems in its batch)."""
import numpy as np
import pytest

from mysph_gb300 import params as P
from mysph_gb300 import serve
from mysph_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [P.PREC_MIXED, P.PREC_FP64])
def test_served_results_equal_alone(gpu, precision):
    reqs = serve.poisson_requests(8, rate=400.0, seed=5, n_lo=800, n_hi=6000, s_lo=20, s_hi=90)
    srv = serve.Server(precision=precision, real_capacity=60_000, wall_capacity=30_000, max_instances=8)
    try:
        stats = srv.run(reqs, chunk=16)
    finally:
        srv.close()
    assert stats["requests"] == 8 and stats["p99_tts_s"] >= stats["p50_tts_s"] > 0
    # requests overlapped on the device
    spans = sorted((r.admitted, r.done) for r in reqs)
    assert any(b[0] < a[1] for a, b in zip(spans, spans[1:]))
    for r in reqs:
        with GpuSolver.from_blocks(r.case) as s:
            s.advance(r.steps)
            for f, v in r.result.items():
                assert np.array_equal(v, s.field(f)[: r.case.n_real]), (r.rid, r.kind, f)


def test_admission_waits_for_capacity(gpu):
    reqs = serve.poisson_requests(4, rate=1000.0, seed=9, n_lo=3000, n_hi=3500, s_lo=10, s_hi=12,
                                  kinds=("dam_break",))
    srv = serve.Server(precision=P.PREC_MIXED, real_capacity=4000, wall_capacity=20_000, max_instances=4)
    try:
        stats = srv.run(reqs, chunk=4)
    finally:
        srv.close()
    # only one request fits at a time: admissions are serialised
    ordered = sorted(reqs, key=lambda r: r.admitted)
    for a, b in zip(ordered, ordered[1:]):
        assert b.admitted >= a.done - 1e-9
    assert stats["requests"] == 4


def test_async_advance_of_two_contexts(gpu):
    """sph_advance_async on two contexts queued back to back, then sph_sync
    on each, gives the same state as sph_advance on each alone, bit for bit,
    and the same Courant statistics."""
    from mysph_gb300 import cases
    from tests.helpers import perturb
    a_case = perturb(cases.dam_break_2d(dx=0.04), seed=91, v_amp=0.2)
    b_case = perturb(cases.dam_break_3d(dx=0.05), seed=92, v_amp=0.2)
    with GpuSolver(a_case) as a, GpuSolver(b_case) as b, GpuSolver(a_case) as ra, GpuSolver(b_case) as rb:
        for k in (1, 9, 6):
            a.advance_async(k)
            b.advance_async(k)
            ca, cb = a.sync(), b.sync()
            assert ca == ra.advance(k) and cb == rb.advance(k)
        for s, r in ((a, ra), (b, rb)):
            for f in ("X", "V", "RHO", "E", "P"):
                assert np.array_equal(s.field(f), r.field(f)), f
