"""Lanes per target of the FP64 passes A and B (SPH_OPT_LANES).

With L lanes a target's neighbours are dealt round-robin, in the walk's
order, over L lanes of a warp, and the L partial sums are added by a fixed
butterfly.  Bars: module outputs and the state after one leap-frog step
within 1e-10 relative L2 of the FP64 oracle, and after up to 20 steps within
1e-8 (the chaotic cases over the steps test_gpu_parity uses); neighbour
counts equal to the oracle's; the same bits from two contexts, and alone and
in a batch, for one L; the forms the option leaves at one lane (SPH = 1,
artificial heat, mixed precision) equal to L = 1 bit for bit; values other
than 1, 2, 4, 8, 16 and 32 rejected.
"""
import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300.solver import GpuBatch, GpuSolver
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import fsi_block_3d, perturb, two_fluid_dam_break, with_heat

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-10
TOL_DRIFT = 1e-8


def _flags(c, flags):
    c.params = c.params.copy()
    c.params.flags |= flags
    return c


def _edge():
    """12 particles: a partial warp, a State = -1 particle, a fixed one."""
    c = perturb(cases.dam_break_2d(dx=0.1, width=0.3, height=0.4), seed=5, v_amp=0.2)
    c.state[3] = -1
    c.boundary[5] = 1
    return c


CASES = {
    "dam2d": lambda: perturb(cases.dam_break_2d(), seed=11, v_amp=0.3, x_frac=0.2),
    "dam3d": lambda: perturb(cases.dam_break_3d(dx=0.03), seed=12, v_amp=0.3, x_frac=0.2),
    "gate": lambda: perturb(cases.gate_2d(dx=0.0025), seed=13, v_amp=0.05, x_frac=0.1),
    "fsi3d": lambda: fsi_block_3d(seed=20),
    "dam2d_xsph": lambda: _flags(perturb(cases.dam_break_2d(), seed=17, v_amp=0.3, x_frac=0.2),
                                 P.F_AVER_VELOCITY),
    "multiphase": lambda: two_fluid_dam_break(seed=22),
    "edge": _edge,
}
DRIFT_STEPS = {"gate": 3, "fsi3d": 3, "edge": 5}
STATE = ("X", "V", "RHO", "E", "P", "DISP", "SHEAR", "DVDT", "DRHODT", "DEDT", "DIVV", "AVER")


def _solver(c, lanes, params=None):
    s = GpuSolver(c, params=params)
    s.set_option(P.OPT_LANES, lanes)
    return s


@pytest.mark.parametrize("lanes", [2, 4, 8, 32])
@pytest.mark.parametrize("name", list(CASES))
def test_lanes_step_parity(gpu, name, lanes):
    c = CASES[name]()
    nr = c.n_real
    # the edge case is held to the one-lane path (its rates to the oracle in
    # test_lanes_module_parity's form below)
    o = Oracle(c) if name != "edge" else None
    with _solver(c, lanes) as s, GpuSolver(c) as one:
        if o is not None:
            o.step()
        s.single_step()
        one.single_step()
        for key in STATE:
            got = s.field(key)[:nr]
            if o is not None:
                assert rel_l2(got, o.field(key)[:nr]) <= TOL_STEP, (key, lanes)
            assert rel_l2(got, one.field(key)[:nr]) <= TOL_STEP, (key, lanes)
        assert np.array_equal(s.field("NNEIGH")[:nr], one.field("NNEIGH")[:nr])
        ns = DRIFT_STEPS.get(name, 20)
        ref = o if o is not None else one
        mx_o, mean_o = ref.advance(ns)
        mx_g, mean_g = s.advance(ns)
        for key in ("X", "V", "RHO", "E", "P", "SHEAR"):
            assert rel_l2(s.field(key)[:nr], ref.field(key)[:nr]) <= TOL_DRIFT, (key, lanes)
        assert mx_g == pytest.approx(mx_o, rel=1e-8)
        assert mean_g == pytest.approx(mean_o, rel=1e-8)


@pytest.mark.parametrize("name", ["dam2d", "gate", "fsi3d", "edge"])
def test_lanes_module_parity(gpu, name):
    """The module calls (sph_internal_force, sph_arti_visc, ...) run the same
    passes, so they take the option too."""
    c = CASES[name]()
    nr = c.n_real
    o = Oracle(c)
    o.rates()
    with _solver(c, 4) as s:
        s.nnps()
        got = {"DRHODT": s.con_density()}
        got["IN_DVDT"], got["IN_DEDT"], got["DSDT"] = s.internal_force()
        got["AV_DVDT"], got["AV_DEDT"] = s.arti_visc()
        got["EX_DVDT"] = s.external_force()
        got["DVDT"], _, got["DEDT"] = s.rates()
    prm = c.params
    for key, val in got.items():
        if name == "edge" and key != "DVDT":   # the rate test_edge_cases holds
            continue
        if key == "DSDT" and not np.any(np.abs(c.type) > 100):
            continue
        if key == "EX_DVDT" and not (prm.flags & (P.F_EXT_FORCE | P.F_DUMMY | P.F_GRAVITY)):
            continue
        if key in ("AV_DVDT", "AV_DEDT") and not (prm.flags & P.F_ARTI_VISC):
            continue
        assert rel_l2(val, o.field(key)[:nr]) <= TOL_STEP, key


@pytest.mark.parametrize("lanes", [4, 8])
def test_lanes_deterministic_and_batch_equals_alone(gpu, lanes):
    members = [cases.ensemble_member(sp) for sp in cases.ensemble_specs(count=3, seed=31, n_lo=300, n_hi=3000)]
    members.append(perturb(cases.dam_break_2d(dx=0.05), seed=32, v_amp=0.2))
    steps = 12
    alone = []
    for m in members:
        with _solver(m, lanes) as a, _solver(m, lanes) as b:
            a.advance(steps)
            b.advance(steps)
            fa = {k: a.field(k) for k in ("X", "V", "RHO", "E")}
            for k, v in fa.items():
                assert np.array_equal(v, b.field(k)), k
            alone.append(fa)
    base = members[0].params.copy()
    nr = sum(m.n_real for m in members)
    nw = sum(m.n_wall for m in members)
    with GpuBatch(base, 4, nr + 100, nw + 100) as bt:
        bt.set_option(P.OPT_LANES, lanes)
        ids = [bt.add(m) for m in members]
        bt.advance(steps)
        for k, want in zip(ids, alone):
            for f, v in want.items():
                assert np.array_equal(bt.field(k, f), v), (k, f)


@pytest.mark.parametrize("form", ["sph1", "heat", "mixed"])
def test_lanes_leave_other_forms_alone(gpu, form):
    c = perturb(cases.dam_break_2d(dx=0.04), seed=41, v_amp=0.3, x_frac=0.2)
    prm = c.params.copy()
    if form == "sph1":
        prm.pa_sph = 1
    elif form == "heat":
        c = with_heat(c, seed=42)
        prm = c.params.copy()
    else:
        prm.precision = P.PREC_MIXED
    with _solver(c, 8, prm) as s, GpuSolver(c, params=prm) as one:
        s.advance(5)
        one.advance(5)
        for k in ("X", "V", "RHO", "E"):
            assert np.array_equal(s.field(k), one.field(k)), (form, k)


def test_lanes_option_values(gpu):
    c = cases.dam_break_2d(dx=0.1, width=0.3, height=0.4)
    with GpuSolver(c) as s:
        for bad in (0, 3, 5, 64, -1, 2.5):
            with pytest.raises(Exception):
                s.set_option(P.OPT_LANES, bad)
        for ok in (1, 2, 4, 8, 16, 32):
            s.set_option(P.OPT_LANES, ok)


def test_tune_lanes_keeps_the_state(gpu):
    """GpuSolver.tune_lanes times the settings on copies of the state, sets
    the fastest and leaves the context's own state where it was."""
    c = perturb(cases.dam_break_2d(dx=0.04), seed=43, v_amp=0.3, x_frac=0.2)
    with GpuSolver(c) as s, GpuSolver(c) as ref:
        s.advance(4)
        ref.advance(4)
        before = {k: s.field(k) for k in ("X", "V", "RHO", "E")}
        best = s.tune_lanes(steps=5, choices=(1, 4))
        assert best in (1, 4)
        for k, v in before.items():
            assert np.array_equal(s.field(k), v), k
        # stepping on gives the bits of a context set to the same lanes
        ref.set_option(P.OPT_LANES, best)
        s.advance(3)
        ref.advance(3)
        for k in ("X", "V", "RHO", "E"):
            assert np.array_equal(s.field(k), ref.field(k)), k
