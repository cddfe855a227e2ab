"""Batches of independent systems (sph_batch_*).

A system advanced inside a batch gives bit-for-bit the state it gives alone:
within one instance the cell sort, the neighbour order and every operation
are those of a plain context, so the test compares with == (relative L2 of
0).  Adding and removing systems between steps leaves the others unchanged.
"""
import ctypes

import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300.solver import GpuBatch, GpuSolver
from tests.helpers import perturb

pytestmark = pytest.mark.gpu

FIELDS = ("X", "V", "RHO", "E", "P")


def _members():
    specs = cases.ensemble_specs(count=5, seed=7, n_lo=300, n_hi=3000)
    out = [cases.ensemble_member(s) for s in specs]
    out.append(perturb(cases.dam_break_2d(dx=0.05), seed=3, v_amp=0.2))
    return out


def _alone(case, steps, prm=None):
    with GpuSolver(case, params=prm) as s:
        s.advance(steps)
        return {k: s.field(k) for k in FIELDS}


def _batch_for(members, prm=None):
    base = members[0].params.copy()
    if prm is not None:
        base.precision = prm
    nr = sum(m.n_real for m in members)
    nw = sum(m.n_wall for m in members)
    return GpuBatch(base, len(members) + 2, nr + 5000, nw + 5000)


@pytest.mark.parametrize("precision", [P.PREC_FP64, P.PREC_MIXED])
def test_batch_equals_alone(gpu, precision):
    members = _members()
    steps = 30
    with _batch_for(members, precision) as b:
        ids = []
        for m in members:
            prm = m.params.copy()
            prm.precision = precision
            ids.append(b.add(m, params=prm))
        b.advance(steps)
        for m, k in zip(members, ids):
            prm = m.params.copy()
            prm.precision = precision
            want = _alone(m, steps, prm)
            for f in FIELDS:
                assert np.array_equal(b.field(k, f), want[f]), (k, f)
            inf = b.info(k)
            assert inf["step"] == steps
            assert inf["time"] == pytest.approx(steps * m.params.dt, rel=1e-12)


def test_batch_add_remove_between_steps(gpu):
    members = _members()
    a, c, late = members[0], members[1], members[2]
    with _batch_for(members) as b:
        ka = b.add(a)
        kc = b.add(c)
        b.advance(10)
        b.remove(kc)
        with pytest.raises(Exception):
            b.field(kc, "X")
        kl = b.add(late)      # joins while `a` is mid-run: its own first step
        b.advance(15)
        want_a = _alone(a, 25)
        want_l = _alone(late, 15)
        for f in FIELDS:
            assert np.array_equal(b.field(ka, f), want_a[f]), f
            assert np.array_equal(b.field(kl, f), want_l[f]), f
        assert b.info(kl)["step"] == 15 and b.info(ka)["step"] == 25


def test_batch_capacity(gpu):
    m = _members()[0]
    with GpuBatch(m.params, 1, m.n_real, m.n_wall) as b:
        b.add(m)
        cap = b.capacity()
        assert cap["free_slots"] == 0 and cap["free_real"] == 0
        with pytest.raises(Exception) as ei:
            b.add(m)
        assert getattr(ei.value, "status", None) == P.SPH_E_NOMEM
        # arrays in one system's upload order are read per instance
        out = np.empty((m.n_real + m.n_wall) * m.dim)
        with pytest.raises(Exception) as ei:
            b._call("sph_get_field", P.FIELD["X"], out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert getattr(ei.value, "status", None) == P.SPH_E_UNSUPPORTED


def test_removed_walls_leave_reused_slot(gpu):
    """A slot freed by a removal and reused at once reads only the new
    system's walls (the old walls stay in the wall region until compaction)."""
    members = _members()
    a, c = members[3], members[4]
    with _batch_for(members) as b:
        ka = b.add(a)
        kc = b.add(c)
        b.advance(2)
        b.remove(kc)
        kn = b.add(a)
        assert kn == kc
        x = b.field(kn, "X")
        assert np.array_equal(x, np.asarray(a.arrays()[0]).reshape(-1, a.dim))
        assert np.array_equal(b.field(kn, "TYPE"), a.arrays()[8].astype(np.float64))


@pytest.mark.parametrize("precision", [P.PREC_FP64, P.PREC_DF64])
def test_batch_equals_alone_3d(gpu, precision):
    """3-D systems, whose lattice targets fill their neighbour lists (56 of 88
    entries) and whose targets near the walls run them mid-walk: each lane's
    pair order, hence its sums, must not depend on the other systems' targets
    in its warp."""
    members = [perturb(cases.dam_break_3d(dx=dx, block=(0.3, 0.2, 0.3), box=(0.8, 0.4, 0.5)),
                       seed=s, v_amp=0.3, x_frac=0.2) for dx, s in ((0.03, 81), (0.025, 82), (0.035, 83))]
    steps = 12
    with _batch_for(members, precision) as b:
        ids = []
        for m in members:
            prm = m.params.copy()
            prm.precision = precision
            ids.append(b.add(m, params=prm))
        b.advance(steps)
        for m, k in zip(members, ids):
            prm = m.params.copy()
            prm.precision = precision
            want = _alone(m, steps, prm)
            for f in FIELDS:
                assert np.array_equal(b.field(k, f), want[f]), (k, f)


def test_batch_cell_space_above_2_24(gpu):
    """Two systems whose cell grids add up to more than 2^24 = 16,777,216
    cells (each about 10 M cells, from a user-given domain): the cell-start
    scan then needs a second level of block partials.  Each system still
    equals itself run alone, bit for bit."""
    members = []
    for seed in (81, 82):
        m = perturb(cases.dam_break_2d(dx=0.1), seed=seed, v_amp=0.2)
        m.params = m.params.copy()
        for a in range(2):
            m.params.domain_lo[a] = -380.0
            m.params.domain_hi[a] = 380.0
        members.append(m)
    steps = 4
    with _batch_for(members) as b:
        ids = [b.add(m) for m in members]
        cs = 2.0 * float(members[0].h[0]) * (1.0 + 1e-9)   # cell = 2 h_max (cubic spline)
        per = int(np.ceil(760.0 / cs)) ** 2
        assert per < (1 << 24) - 2 and 2 * per > (1 << 24)
        b.advance(steps)
        for m, k in zip(members, ids):
            want = _alone(m, steps)
            for f in FIELDS:
                assert np.array_equal(b.field(k, f), want[f]), (k, f)
