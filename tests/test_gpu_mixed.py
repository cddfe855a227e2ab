"""Mixed precision (SPH_PREC_MIXED): FP32 kernel weights, EOS and pair forces
with Kahan-compensated sums; FP64 positions and leap-frog update.

Bars, stated per field:
- rates of one step against the FP64 oracle: relative L2 <= 1e-4;
- after a run (the 2-D dam break of 5,000 particles over its 1,000 steps, a
  3-D dam break over 300 steps, the elastic gate over 200 steps) density and
  velocity against the FP64 GPU path: relative L2 <= 1e-3.
The FP64 GPU path itself equals the oracle (tests/test_gpu_parity.py).
"""
import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300.solver import GpuSolver
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import fsi_block_3d, perturb, plastic_block, two_fluid_dam_break

pytestmark = pytest.mark.gpu

TOL_RATES = 1e-4
TOL_RUN = 1e-3


def mixed(case):
    prm = case.params.copy()
    prm.precision = P.PREC_MIXED
    return prm


RATE_CASES = {
    "dam2d": lambda: perturb(cases.dam_break_2d(), seed=31, v_amp=0.3, x_frac=0.2),
    "dam3d": lambda: perturb(cases.dam_break_3d(dx=0.03), seed=32, v_amp=0.3, x_frac=0.2),
    "gate": lambda: perturb(cases.gate_2d(dx=0.0025), seed=33, v_amp=0.05, x_frac=0.1),
    "fsi3d": lambda: fsi_block_3d(seed=35),
    "dam2d_sum_xsph": lambda: _flags(perturb(cases.dam_break_2d(), seed=34, v_amp=0.3, x_frac=0.2),
                                     P.F_SUM_DENSITY | P.F_NORM_DENSITY | P.F_AVER_VELOCITY),
    "multiphase": lambda: two_fluid_dam_break(seed=36),
    # elastic-plastic solids (Mie-Grueneisen 101, aluminium 104); no walls, so
    # the oracle's grid band is widened to cover 2h
    "mg2d": lambda: plastic_block(2, 101, seed=37),
    "mg3d": lambda: plastic_block(3, 101, seed=38, n=8),
    "al3d": lambda: plastic_block(3, 104, seed=39, n=8),
}


def _flags(c, f):
    c.params = c.params.copy()
    c.params.flags |= f
    return c


@pytest.mark.parametrize("name", list(RATE_CASES))
def test_mixed_rates_vs_oracle(gpu, name):
    c = RATE_CASES[name]()
    o = Oracle(c, covering_band=c.name.startswith("plastic"))
    o.rates()
    nr = c.n_real
    with GpuSolver(c, params=mixed(c)) as s:
        s.nnps()
        a, drho, de = s.rates()
        rho, aver = s.field("RHO")[:nr], s.field("AVER")[:nr]
        dsdt = s.field("DSDT")[:nr] if np.any(np.abs(c.type) > 100) else None
    errs = {"DVDT": rel_l2(a, o.field("DVDT")[:nr]), "DRHODT": rel_l2(drho, o.field("DRHODT")[:nr]),
            "DEDT": rel_l2(de, o.field("DEDT")[:nr]), "RHO": rel_l2(rho, o.field("RHO")[:nr])}
    if c.params.flags & P.F_AVER_VELOCITY:
        errs["AVER"] = rel_l2(aver, o.field("AVER")[:nr])
    if dsdt is not None:
        errs["DSDT"] = rel_l2(dsdt, o.field("DSDT")[:nr])
    print(name, errs)
    for k, e in errs.items():
        assert e <= TOL_RATES, (k, e)


@pytest.mark.parametrize("name,maker,steps", [
    ("dam2d", lambda: cases.dam_break_2d(), 1000),
    ("dam3d", lambda: cases.dam_break_3d(dx=0.02), 300),
    ("gate", lambda: cases.gate_2d(dx=0.0025), 200),
    ("dam2d_sum_xsph", lambda: _flags(cases.dam_break_2d(), P.F_SUM_DENSITY | P.F_NORM_DENSITY
                                      | P.F_AVER_VELOCITY), 500),
])
def test_mixed_run_vs_fp64(gpu, name, maker, steps):
    c = maker()
    with GpuSolver(c) as f64, GpuSolver(c, params=mixed(c)) as f32:
        f64.advance(steps)
        f32.advance(steps)
        nr = c.n_real
        errs = {k: rel_l2(f32.field(k)[:nr], f64.field(k)[:nr]) for k in ("RHO", "V", "X", "P")}
    print(name, steps, errs)
    assert errs["RHO"] <= TOL_RUN and errs["V"] <= TOL_RUN, errs


def test_mixed_lattice_neighbor_counts(gpu):
    """On the initial lattice no pair sits near 2h, so the FP32 test of the
    mixed pass finds exactly the FP64 sets' sizes."""
    c = cases.dam_break_3d(dx=0.02)
    with GpuSolver(c) as f64:
        f64.nnps()
        want = f64.neighbor_counts()
    with GpuSolver(c, params=mixed(c)) as s:
        s.nnps()
        s.con_density()
        got = s.field("NNEIGH")[: c.n_real].astype(np.int32)
    assert np.array_equal(got, want)


def test_switch_precision(gpu):
    c = cases.dam_break_2d(dx=0.05)
    with GpuSolver(c) as s:
        s.advance(5)
        prm = c.params.copy()
        prm.precision = P.PREC_MIXED
        s._call("sph_set_params", __import__("ctypes").byref(prm))
        s.advance(5)
        assert np.all(np.isfinite(s.field("V")))
        assert s.info()["step"] == 10


@pytest.mark.parametrize("block,list_len,persistent", [(32, 64, 0), (64, 120, 1), (128, 88, 1), (128, 120, 0)])
def test_launch_knobs_do_not_change_results(gpu, block, list_len, persistent):
    """Block size, list length and the persistent launch form only move the
    points where the warp runs the pair physics, or which block runs a tile
    of targets; every lane keeps its neighbour order, so the state is
    bit-for-bit the same."""
    c = perturb(cases.dam_break_3d(dx=0.04), seed=35, v_amp=0.3, x_frac=0.2)
    with GpuSolver(c, params=mixed(c)) as a, GpuSolver(c, params=mixed(c)) as b:
        b.set_option(P.OPT_BLOCK_SIZE, block)
        b.set_option(P.OPT_LIST_LEN, list_len)
        b.set_option(P.OPT_PERSISTENT, persistent)
        a.advance(6)
        b.advance(6)
        for k in ("X", "V", "RHO", "P"):
            assert np.array_equal(a.field(k), b.field(k)), k


def test_launch_knob_validation(gpu):
    from mysph_gb300._lib import SphError
    c = cases.dam_break_2d(dx=0.1)
    with GpuSolver(c, params=mixed(c)) as s:
        for opt, val in ((P.OPT_BLOCK_SIZE, 96), (P.OPT_BLOCK_SIZE, 256), (P.OPT_LIST_LEN, 40),
                         (P.OPT_LIST_LEN, 72), (P.OPT_PERSISTENT, 2)):
            with pytest.raises(SphError):
                s.set_option(opt, val)
