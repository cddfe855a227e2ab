"""FP64 energy sums (sph_energy): kinetic, internal and gravitational energy
of the real particles, summed on the device in a fixed order.

Bars: equal to the same sums formed in numpy from the downloaded fields
within 1e-13 relative; the same bits on repeated calls and on two contexts
holding the same state; a system of a batch within 1e-14 of itself run alone
(the block partition of the sum differs), and the batch total equal to the
sum of its systems; the mixed-precision form's total within 1e-4 of the FP64
form's after 100 steps.
"""
import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300.solver import GpuBatch, GpuSolver
from tests.helpers import perturb

pytestmark = pytest.mark.gpu

CASES = {
    "dam2d": lambda: perturb(cases.dam_break_2d(dx=0.04), seed=111, v_amp=0.3, x_frac=0.2),
    "dam3d": lambda: perturb(cases.dam_break_3d(dx=0.03), seed=112, v_amp=0.3, x_frac=0.2),
}


def _numpy_energy(s, c):
    nr, dim = c.n_real, c.dim
    x, v = s.field("X")[:nr], s.field("V")[:nr]
    m, e = s.field("MASS")[:nr], s.field("E")[:nr]
    k = 0.5 * np.sum(m * np.sum(v * v, axis=1))
    u = np.sum(m * e)
    g = -np.sum(m * c.params.gravity * x[:, dim - 1]) if c.params.flags & P.F_GRAVITY else 0.0
    return k, u, g


@pytest.mark.parametrize("name", list(CASES))
def test_energy_sums(gpu, name):
    c = CASES[name]()
    with GpuSolver(c) as a, GpuSolver(c) as b:
        a.advance(7)
        b.advance(7)
        ea, eb = a.energy(), b.energy()
        assert ea == eb and a.energy() == ea        # fixed summation order
        k, u, g = _numpy_energy(a, c)
        assert ea["kinetic"] == pytest.approx(k, rel=1e-13)
        assert ea["internal"] == pytest.approx(u, rel=1e-13, abs=1e-300)
        assert ea["gravitational"] == pytest.approx(g, rel=1e-13)
        assert ea["total"] == (ea["kinetic"] + ea["internal"]) + ea["gravitational"]
        assert ea["kinetic"] > 0 and ea["gravitational"] != 0


def test_energy_of_batch_systems(gpu):
    members = [perturb(cases.dam_break_2d(dx=0.05), seed=s, v_amp=0.2) for s in (113, 114, 115)]
    nr = sum(m.n_real for m in members)
    nw = sum(m.n_wall for m in members)
    with GpuBatch(members[0].params, 4, nr + 10, nw + 10) as b:
        ids = [b.add(m) for m in members]
        b.advance(5)
        per = [b.energy(k) for k in ids]
        tot = b.energy(-1)
        for m, k, e in zip(members, ids, per):
            with GpuSolver(m) as s:
                s.advance(5)
                alone = s.energy()
            for f in ("kinetic", "internal", "gravitational", "total"):
                assert e[f] == pytest.approx(alone[f], rel=1e-14, abs=1e-300), (k, f)
        for f in ("kinetic", "gravitational", "total"):
            assert tot[f] == pytest.approx(sum(e[f] for e in per), rel=1e-14)


def test_mixed_energy_close_to_fp64(gpu):
    c = CASES["dam2d"]()
    prm = c.params.copy()
    prm.precision = P.PREC_MIXED
    with GpuSolver(c) as f64, GpuSolver(c, params=prm) as mix:
        f64.advance(100)
        mix.advance(100)
        e64, em = f64.energy(), mix.energy()
    assert em["total"] == pytest.approx(e64["total"], rel=1e-4)
    assert em["kinetic"] == pytest.approx(e64["kinetic"], rel=1e-3)
