"""sph_step_host: the drop-in form of leap_frog's loop for a host that owns
the particle arrays (the call bench.py's `e2e` times).

Each call copies the real particles' x, v, rho, e (and the deviatoric
stress) in from host memory, in the uploaded order, steps on the device and
copies the same arrays back.  The tests drive a context only through that
call, with pageable and with pinned host arrays, and check the arrays it
hands back: bit for bit against the same steps through sph_advance, and
within 1e-10 relative L2 of the FP64 oracle after one step.  A host that
changes its arrays between calls steers the next step.
"""
import ctypes as C

import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300.solver import GpuSolver
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import perturb

pytestmark = pytest.mark.gpu

CASES = {
    "dam2d": lambda: perturb(cases.dam_break_2d(dx=0.04), seed=101, v_amp=0.3, x_frac=0.2),
    "dam3d": lambda: perturb(cases.dam_break_3d(dx=0.04), seed=102, v_amp=0.3, x_frac=0.2),
    "gate": lambda: perturb(cases.gate_2d(dx=0.005), seed=103, v_amp=0.05, x_frac=0.1),
}


def _host_arrays(c, pinned):
    nr, dim = c.n_real, c.dim
    vals = {"x": c.x[:nr].ravel(), "v": c.v[:nr].ravel(), "rho": c.rho[:nr], "e": c.e[:nr]}
    if c.shear is not None:
        vals["shear"] = c.shear[:nr].ravel()
    out = {}
    for k, a in vals.items():
        if pinned:
            import torch
            t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
            t.numpy()[:] = a
            out[k] = (t, t.numpy())
        else:
            arr = np.ascontiguousarray(a, dtype=np.float64).copy()
            out[k] = (arr, arr)
    return out


def _step_host(s, arrs, nsteps):
    p = lambda k: arrs[k][1].ctypes.data_as(C.POINTER(C.c_double)) if k in arrs else None
    s._call("sph_step_host", int(nsteps), p("x"), p("v"), p("rho"), p("e"), p("shear"))


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("name", list(CASES))
def test_step_host_equals_advance_and_oracle(gpu, name, pinned):
    c = CASES[name]()
    nr, dim = c.n_real, c.dim
    arrs = _host_arrays(c, pinned)
    o = Oracle(c)
    with GpuSolver(c) as h, GpuSolver(c) as r:
        _step_host(h, arrs, 1)
        r.single_step()
        o.step()
        got = {"X": arrs["x"][1].reshape(nr, dim), "V": arrs["v"][1].reshape(nr, dim),
               "RHO": arrs["rho"][1], "E": arrs["e"][1]}
        if "shear" in arrs:
            got["SHEAR"] = arrs["shear"][1].reshape(nr, dim * dim)
        for k, v in got.items():
            assert np.array_equal(v, r.field(k)[:nr]), k
            assert rel_l2(v, o.field(k)[:nr]) <= 1e-10, k
        # several calls, then a multi-step call: still the bits of sph_advance
        for n in (1, 1, 3):
            _step_host(h, arrs, n)
            r.advance(n)
        for k, v in got.items():
            assert np.array_equal(v, r.field(k)[:nr]), k


def test_step_host_reads_the_host_arrays(gpu):
    """A change the host makes to its arrays between calls is what the next
    step starts from: equal to setting the same fields on the device."""
    c = CASES["dam2d"]()
    nr, dim = c.n_real, c.dim
    arrs = _host_arrays(c, False)
    with GpuSolver(c) as h, GpuSolver(c) as r:
        _step_host(h, arrs, 2)
        r.advance(2)
        v = arrs["v"][1].reshape(nr, dim)
        v[:, 0] += 0.01
        rv = r.field("V")
        rv[:nr, 0] += 0.01
        r.set_field("V", rv)
        _step_host(h, arrs, 2)
        r.advance(2)
        assert np.array_equal(arrs["v"][1].reshape(nr, dim), r.field("V")[:nr])
        assert np.array_equal(arrs["x"][1].reshape(nr, dim), r.field("X")[:nr])
