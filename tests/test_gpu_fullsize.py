"""GPU parity at the full sizes of the measured workloads.

The 3-D dam break at dx = 4 mm (1,687,500 real and 1,024,008 wall particles,
the bench workload) and the elastic gate at dx = 0.5 mm (322,000 real
particles) each take two leap-frog steps on the GPU, through the C ABI, and
in the OpenMP build of the oracle.  That build forms every target's sums in
the reference's serial order (threads split the targets, not a target's
neighbours) and rounds every operation as the serial checker does, so it is
the same FP64 oracle, only faster.  Bar: identical neighbour sets, compared
as CSR arrays sorted within each row, and every state field within 1e-10
relative L2 after each step.  Both cases are perturbed so that the
artificial viscosity, the strain rate and the guard band of the distance
test all run.
"""
import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300.solver import GpuSolver
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import bggs_band_covers, perturb

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-10

FULL = {
    "dam3d_dx4mm": lambda: perturb(cases.dam_break_3d(), seed=71, v_amp=0.3, x_frac=0.2),
    "gate_dx0p5mm": lambda: perturb(cases.gate_2d(), seed=72, v_amp=0.05, x_frac=0.1),
}


def sorted_rows(off, lst):
    """CSR rows as one array of (row, column) keys, sorted: equal arrays
    mean equal neighbour sets row by row."""
    off = np.asarray(off, dtype=np.int64)
    seg = np.repeat(np.arange(len(off) - 1, dtype=np.int64), np.diff(off))
    return np.sort(seg * np.int64(1 << 32) + np.asarray(lst, dtype=np.int64))


@pytest.mark.parametrize("name", list(FULL))
def test_full_size_step_parity(gpu, name):
    c = FULL[name]()
    assert bggs_band_covers(c)
    nr = c.n_real
    o = Oracle(c, omp=True)
    o.bggs()
    off_o, lst_o = o.neighbors()
    with GpuSolver(c) as s:
        s.nnps()
        off_g, lst_g = s.neighbor_lists()
        assert np.array_equal(off_g, off_o)
        assert np.array_equal(sorted_rows(off_g, lst_g), sorted_rows(off_o, lst_o))
        del off_g, lst_g, off_o, lst_o
        for step in (1, 2):
            o.step()
            s.single_step()
            for key in ("X", "V", "RHO", "E", "P", "SHEAR", "DVDT", "DRHODT", "DEDT", "DIVV"):
                if key == "SHEAR" and c.shear is None:
                    continue
                err = rel_l2(s.field(key)[:nr], o.field(key)[:nr])
                assert err <= TOL_STEP, (step, key, err)
