"""Smoothing-length evolution (SLE = 1, 2; hsml.f90:8-38) against the
oracle; the hash cell is given room for the growing h with
sph_params.cell_size, and outgrowing it is reported as SPH_E_RANGE."""
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300._lib import SphError
from mysph_gb300.solver import GpuSolver
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import perturb

pytestmark = pytest.mark.gpu


def _sle(sle, cell_factor):
    c = perturb(cases.dam_break_2d(dx=0.04), seed=70 + sle, v_amp=0.3, x_frac=0.2)
    c.params = c.params.copy()
    c.params.sle = sle
    c.params.cell_size = cell_factor * c.meta["dx"]
    return c


@pytest.mark.parametrize("sle,cell_factor", [(1, 4.5), (2, 3.0)])
def test_sle_parity(gpu, sle, cell_factor):
    c = _sle(sle, cell_factor)
    o = Oracle(c, covering_band=True)
    with GpuSolver(c) as s:
        o.step()
        s.single_step()
        for key in ("X", "V", "RHO", "H", "P", "DVDT"):
            err = rel_l2(s.field(key)[: c.n_real], o.field(key)[: c.n_real])
            assert err <= 1e-10, (key, err)
        o.advance(10)
        s.advance(10)
        for key in ("X", "V", "RHO", "H"):
            err = rel_l2(s.field(key)[: c.n_real], o.field(key)[: c.n_real])
            assert err <= 1e-8, (key, err)


def test_sle_outgrowing_the_cell_is_reported(gpu):
    c = _sle(1, 2.5)                  # h -> ~2 dx needs cells of ~4 dx
    with GpuSolver(c) as s:
        with pytest.raises(SphError) as ei:
            s.single_step()
        assert ei.value.status == P.SPH_E_RANGE
