"""State snapshots (sph_state_save / sph_state_load): a context resumed from
a snapshot continues bit for bit like the original, for the FP64 and mixed
paths, solids, summation density and batches."""
import numpy as np
import pytest

from mysph_gb300 import cases
from mysph_gb300 import params as P
from mysph_gb300._lib import SphError
from mysph_gb300.solver import GpuBatch, GpuSolver
from tests.helpers import perturb

pytestmark = pytest.mark.gpu

FIELDS = ("X", "V", "RHO", "E", "P", "DISP")


def _flags(c, f, precision=P.PREC_FP64):
    c.params = c.params.copy()
    c.params.flags |= f
    c.params.precision = precision
    return c


CASES = {
    "dam2d_fp64": lambda: perturb(cases.dam_break_2d(dx=0.04), seed=41, v_amp=0.3, x_frac=0.2),
    "dam2d_mixed": lambda: _flags(perturb(cases.dam_break_2d(dx=0.04), seed=42, v_amp=0.3, x_frac=0.2),
                                  0, P.PREC_MIXED),
    "gate_mixed": lambda: _flags(perturb(cases.gate_2d(dx=0.005), seed=43, v_amp=0.05, x_frac=0.1),
                                 0, P.PREC_MIXED),
    "dam3d_sumnorm": lambda: _flags(perturb(cases.dam_break_3d(dx=0.05), seed=44, v_amp=0.3, x_frac=0.2),
                                    P.F_SUM_DENSITY | P.F_NORM_DENSITY),
}


@pytest.mark.parametrize("name", list(CASES))
def test_resume_is_bitwise(gpu, name):
    c = CASES[name]()
    fields = FIELDS + (("SHEAR",) if np.any(np.abs(c.type) > 100) else ())
    with GpuSolver(c) as s:
        s.advance(7)
        blob = s.save_state()
        mx0, mean0 = s.advance(9)
        want = {k: s.field(k) for k in fields}
        info0 = s.info()
    with GpuSolver.from_state(blob) as r:
        assert r.info()["step"] == 7
        mx1, mean1 = r.advance(9)
        for k in fields:
            assert np.array_equal(r.field(k), want[k]), k
        assert r.info() == info0
        assert (mx1, mean1) == (mx0, mean0)


def test_resume_batch(gpu):
    specs = cases.ensemble_specs(count=3, seed=9, n_lo=300, n_hi=2000)
    ms = [cases.ensemble_member(sp) for sp in specs]
    nr = sum(m.n_real for m in ms)
    nw = sum(m.n_wall for m in ms)
    with GpuBatch(ms[0].params, 4, nr + 100, nw + 100) as b:
        ids = [b.add(m) for m in ms[:2]]
        b.advance(5)
        b.remove(ids[0])
        ids.append(b.add(ms[2]))
        b.advance(3)
        blob = b.save_state()
        b.advance(6)
        want = {k: {f: b.field(k, f) for f in FIELDS} for k in ids[1:]}
    with GpuBatch.from_state(blob) as r:
        assert sorted(r.slots()) == sorted(ids[1:])
        r.advance(6)
        for k in ids[1:]:
            for f in FIELDS:
                assert np.array_equal(r.field(k, f), want[k][f]), (k, f)


def test_bad_snapshot_is_rejected(gpu):
    c = cases.dam_break_2d(dx=0.1)
    with GpuSolver(c) as s:
        blob = bytearray(s.save_state())
    blob[0] ^= 0xFF                      # magic
    with pytest.raises(SphError):
        GpuSolver.from_state(bytes(blob))
    blob[0] ^= 0xFF
    with pytest.raises(SphError):
        GpuSolver.from_state(bytes(blob[: len(blob) // 2]))   # truncated
