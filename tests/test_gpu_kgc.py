"""Kernel gradient correction (kernelGradientCorrection.f90:8-51) on the GPU
against the oracle.  Thin solids trip the reference's BGGS band deficit, so
the oracle runs with a covering band (the exact r < 2h sets the GPU uses)."""
import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300._lib import SphError
from mysph_gb300.solver import GpuSolver
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import perturb

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-10
TOL_DRIFT = 1e-8


def _kgc(c):
    c.params = c.params.copy()
    c.params.flags |= P.F_KERNEL_CORRECTION
    return c


def _solid_block_3d():
    c = perturb(cases.dam_break_3d(dx=0.05), seed=52, v_amp=0.2, x_frac=0.1)
    c.type[: c.n_real] = 102
    c.shear = np.zeros((c.n, 9))
    c.params = c.params.copy()
    c.params.flags &= ~(P.F_GRAVITY | P.F_DUMMY | P.F_EXT_FORCE)
    c.params.add_material(**P.linear_solid(102, 1000.0, P.f32(2e7), P.f32(4.27e6)))
    cs = (P.f32(2e7) / 1000.0) ** 0.5          # solid sound speed, and a time step for it
    c.c = c.c.copy()
    c.c[: c.n_real] = cs
    c.params.dt = 0.2 * float(c.h[0]) / cs
    return _kgc(c)


CASES = {
    "cantilever": lambda: _kgc(perturb(cases.cantilever_2d(dx=2e-3, length=0.04, thickness=0.01),
                                       seed=51, v_amp=0.5, x_frac=0.1)),
    "block3d": _solid_block_3d,
}


@pytest.mark.parametrize("name", list(CASES))
def test_kgc_parity(gpu, name):
    c = CASES[name]()
    o = Oracle(c, covering_band=True)
    with GpuSolver(c) as s:
        o.step()
        s.single_step()
        for key in ("X", "V", "RHO", "E", "P", "SHEAR", "DVDT", "DRHODT", "DEDT", "DIVX", "DIVV"):
            err = rel_l2(s.field(key)[: c.n_real], o.field(key)[: c.n_real])
            assert err <= TOL_STEP, (key, err)
        o.advance(10)
        s.advance(10)
        for key in ("X", "V", "RHO", "SHEAR"):
            err = rel_l2(s.field(key)[: c.n_real], o.field(key)[: c.n_real])
            assert err <= TOL_DRIFT, (key, err)


def test_kgc_position_divergence_is_dim(gpu):
    c = CASES["cantilever"]()
    with GpuSolver(c) as s:
        s.nnps()
        dx, _ = s.divergence()
    assert np.max(np.abs(dx - 2.0)) < 1e-12


def test_kgc_needs_solid_targets(gpu):
    c = _kgc(cases.dam_break_2d(dx=0.1))
    with pytest.raises(SphError) as ei:
        GpuSolver(c)
    assert ei.value.status == P.SPH_E_UNSUPPORTED
    prm = CASES["cantilever"]().params.copy()
    prm.precision = P.PREC_MIXED
    with pytest.raises(SphError):
        GpuSolver(CASES["cantilever"](), params=prm)
