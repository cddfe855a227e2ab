"""SPH_PREC_DF64: the pair physics in double-float arithmetic on the FP32
pipes, held to the FP64 path's bar against the oracle: identical neighbour
sets (the FP64 test is unchanged), 1e-10 relative L2 after one step and for
every module output, 1e-8 after 20 steps."""
import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300._lib import SphError
from mysph_gb300.solver import GpuBatch, GpuSolver
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import csr_sets, perturb

pytestmark = pytest.mark.gpu


def _df(c):
    prm = c.params.copy()
    prm.precision = P.PREC_DF64
    return prm


def _flags(c, f):
    c.params = c.params.copy()
    c.params.flags |= f
    return c


CASES = {
    "dam2d": lambda: perturb(cases.dam_break_2d(), seed=91, v_amp=0.3, x_frac=0.2),
    "dam2d_rest": lambda: cases.dam_break_2d(),
    "dam3d": lambda: perturb(cases.dam_break_3d(dx=0.03), seed=92, v_amp=0.3, x_frac=0.2),
    "ref_dam": lambda: cases.reference_dam_break(),
    "dam2d_sum": lambda: _flags(perturb(cases.dam_break_2d(), seed=93, v_amp=0.3, x_frac=0.2),
                                P.F_SUM_DENSITY | P.F_NORM_DENSITY),
    "dam2d_xsph": lambda: _flags(perturb(cases.dam_break_2d(), seed=95, v_amp=0.3, x_frac=0.2),
                                 P.F_AVER_VELOCITY),
    "dam3d_xsph": lambda: _flags(perturb(cases.dam_break_3d(dx=0.03), seed=96, v_amp=0.3, x_frac=0.2),
                                 P.F_SUM_DENSITY | P.F_AVER_VELOCITY),
}


@pytest.mark.parametrize("name", list(CASES))
def test_df64_step_parity(gpu, name):
    c = CASES[name]()
    o = Oracle(c)
    o.bggs()
    want = csr_sets(*o.neighbors())
    with GpuSolver(c, params=_df(c)) as s:
        s.nnps()
        assert csr_sets(*s.neighbor_lists()) == want
        o.step()
        s.single_step()
        keys = ["X", "V", "RHO", "E", "P", "DVDT", "DRHODT", "DEDT", "DIVV"]
        if c.params.flags & P.F_AVER_VELOCITY:
            keys.append("AVER")
        for key in keys:
            err = rel_l2(s.field(key)[: c.n_real], o.field(key)[: c.n_real])
            assert err <= 1e-10, (key, err)
        o.advance(20)
        s.advance(20)
        for key in ("X", "V", "RHO", "E", "P"):
            err = rel_l2(s.field(key)[: c.n_real], o.field(key)[: c.n_real])
            assert err <= 1e-8, (key, err)


def test_df64_module_parity(gpu):
    c = CASES["dam2d"]()
    o = Oracle(c)
    o.rates()
    nr = c.n_real
    with GpuSolver(c, params=_df(c)) as s:
        s.nnps()
        got = {"DRHODT": s.con_density()}
        got["DIVX"], got["DIVV"] = s.divergence()
        got["IN_DVDT"], got["IN_DEDT"], _ = s.internal_force()
        got["AV_DVDT"], got["AV_DEDT"] = s.arti_visc()
        got["EX_DVDT"] = s.external_force()
        got["DVDT"], _, got["DEDT"] = s.rates()
    for k, v in got.items():
        assert rel_l2(v, o.field(k)[:nr]) <= 1e-10, k


@pytest.mark.parametrize("flags", [0, P.F_AVER_VELOCITY])
def test_df64_batch_equals_alone(gpu, flags):
    specs = cases.ensemble_specs(count=3, seed=94, n_lo=300, n_hi=2000)
    ms = [_flags(cases.ensemble_member(sp), flags) for sp in specs]
    base = _df(ms[0])
    with GpuBatch(base, 4, sum(m.n_real for m in ms), sum(m.n_wall for m in ms)) as b:
        ids = [b.add(m, params=_df(m)) for m in ms]
        b.advance(12)
        for k, m in zip(ids, ms):
            with GpuSolver(m, params=_df(m)) as s:
                s.advance(12)
                for f in ("X", "V", "RHO"):
                    assert np.array_equal(b.field(k, f), s.field(f)), (k, f)


def test_df64_scope(gpu):
    g = cases.gate_2d(dx=0.005)
    with pytest.raises(SphError) as ei:
        GpuSolver(g, params=_df(g))
    assert ei.value.status == P.SPH_E_UNSUPPORTED
    for f in (P.F_ARTI_STRESS, P.F_KERNEL_CORRECTION):
        c = _flags(cases.dam_break_2d(dx=0.1), f)
        with pytest.raises(SphError):
            GpuSolver(c, params=_df(c))
