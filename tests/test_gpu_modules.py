"""The last two module procedures of the drop-in boundary on the GPU:
boundary (boundaryCondition.f90:15-45, fixedBoundary) applied to host-side
module sums, and courant_num (courantNumber.f90:7-31)."""
import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300.solver import GpuSolver
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import perturb

pytestmark = pytest.mark.gpu


def test_boundary_after_module_calls(gpu):
    """in + av + ex + as summed on the host in single_step's order, then
    boundary(): the assembled rate of sph_rates, bit for bit, and the oracle's
    within 1e-10; rows with Boundary == 1 are zero."""
    c = perturb(cases.gate_2d(dx=0.0025), seed=61, v_amp=0.05, x_frac=0.1)
    nr = c.n_real
    fixed = c.boundary[:nr] == 1
    assert fixed.any()
    o = Oracle(c)
    o.rates()
    with GpuSolver(c) as s:
        s.nnps()
        a_in, _, _ = s.internal_force()
        a_av, _ = s.arti_visc()
        a_ex = s.external_force()
        a_as = s.artificial_stress()
        total = ((a_in + a_av) + a_ex) + a_as
        got = s.boundary(total)
        assert np.all(got.reshape(nr, -1)[fixed] == 0.0)
        assert np.array_equal(got.reshape(nr, -1)[~fixed], total.reshape(nr, -1)[~fixed])
        a, _, _ = s.rates()
        assert np.array_equal(got, a)
    assert rel_l2(got, o.field("DVDT")[:nr]) <= 1e-10


def test_courant_num_matches_the_step(gpu):
    """courant_num on the state after a step reproduces the step's reported
    maximum, and the formula with the context's dt and alpha / beta."""
    c = perturb(cases.dam_break_2d(), seed=62, v_amp=0.3, x_frac=0.2)
    nr = c.n_real
    with GpuSolver(c) as s:
        mx, _ = s.advance(3)
        h, dv, cc = s.field("H")[:nr], s.field("DIVV")[:nr], s.field("C")[:nr]
        xi = s.courant_num(h, dv, cc)
    assert xi.max() == mx
    p = c.params
    want = p.dt * (h * dv + cc + float(np.float32(1.2)) * (p.cour_alpha * cc + p.cour_beta * h * np.abs(dv))) / h
    np.testing.assert_allclose(xi, want, rtol=1e-15, atol=0)
