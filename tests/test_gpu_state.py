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


# ctypes mirrors of the snapshot's header and instance records (sph_ctx.cu);
# the test checks their sizes against the sizes the snapshot itself records.
import ctypes as C  # noqa: E402


class _Grid(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("inv_cs", C.c_double), ("cs", C.c_double),
                ("nc", C.c_int32 * 3), ("ncells", C.c_int32), ("guard", C.c_float), ("cs_f", C.c_float),
                ("div_m", C.c_uint64 * 2), ("div_l", C.c_int32 * 2)]


class _Inst(C.Structure):
    _fields_ = [("grid", _Grid)] + [(k, C.c_int32) for k in (
        "cell_base", "mat_base", "n_mat", "n_real", "step", "active", "wall_first", "n_wall")] + [
        (k, C.c_double) for k in ("dt", "time", "wall_r0", "contact_delta", "as_dp")] + [
        (k, C.c_float) for k in ("ext_wall_r2", "ext_delta", "wall_r0_f")]


class _Header(C.Structure):
    _fields_ = [("magic", C.c_char * 8)] + [(k, C.c_uint32) for k in (
        "version", "header_bytes", "params_bytes", "inst_bytes", "material_bytes", "reserved")] + [
        ("prm", P.SphParams)] + [(k, C.c_int32) for k in (
            "batch", "max_inst", "has_solid", "mirrors", "dxp", "key_bits")] + [(k, C.c_int64) for k in (
                "capacity", "real_cap", "wall_end", "cell_cap", "pending_remove", "n_real", "n_wall",
                "wall_off", "total_cells", "step")] + [("time", C.c_double), ("payload_bytes", C.c_int64)]


class _InstRec(C.Structure):
    _fields_ = [("I", _Inst), ("prm", P.SphParams), ("n_real", C.c_int64), ("n_wall", C.c_int64),
                ("wall_first", C.c_int64), ("used", C.c_int32), ("reserved", C.c_int32)]


def test_tampered_snapshot_is_rejected(gpu):
    """A snapshot whose header or instance record points outside its own
    ranges (walls, cells, key width, material rows) is refused with
    SPH_E_INVALID before any kernel can index with it."""
    c = cases.dam_break_2d(dx=0.1)
    with GpuSolver(c) as s:
        s.advance(2)
        blob = s.save_state()
    h = _Header.from_buffer_copy(blob)
    assert h.header_bytes == C.sizeof(_Header) and h.inst_bytes == C.sizeof(_Inst)
    off = C.sizeof(_Header)
    rec = _InstRec.from_buffer_copy(blob, off)
    assert rec.used == 1 and rec.n_wall == c.n_wall and rec.I.n_wall == c.n_wall

    def load(b):
        ctx = C.c_void_p()
        buf = C.create_string_buffer(bytes(b), len(b))
        st = gpu.sph_state_load(C.cast(buf, C.c_void_p), len(b), C.byref(ctx))
        if st == 0:
            gpu.sph_destroy(ctx)
        return st

    assert load(blob) == P.SPH_OK

    def with_header(**kw):
        hh = _Header.from_buffer_copy(blob)
        for k, v in kw.items():
            setattr(hh, k, v)
        return bytes(hh) + blob[off:]

    def with_inst(**kw):
        r = _InstRec.from_buffer_copy(blob, off)
        for k, v in kw.items():
            if k.startswith("I_"):
                setattr(r.I, k[2:], v)
            elif k.startswith("nc"):
                r.I.grid.nc[int(k[2])] = v
            elif k.startswith("div_m"):
                r.I.grid.div_m[int(k[5])] = v
            else:
                setattr(r, k, v)
        return blob[:off] + bytes(r) + blob[off + C.sizeof(_InstRec):]

    bad = {
        "key_bits 0": with_header(key_bits=0),
        "key_bits too narrow": with_header(key_bits=1),
        "negative wall count": with_header(n_wall=-1),
        "walls past wall_end": with_inst(n_wall=rec.n_wall + 1000, I_n_wall=rec.n_wall + 1000),
        "walls before wall_off": with_inst(wall_first=-5, I_wall_first=-5),
        "records disagree": with_inst(I_n_wall=rec.n_wall + 1),
        "cells past total": with_inst(I_cell_base=int(h.total_cells)),
        "grid product": with_inst(nc0=rec.I.grid.nc[0] + 1),
        "cell-key divisor": with_inst(div_m0=rec.I.grid.div_m[0] + 1),
        "material rows": with_inst(I_mat_base=8),
        "real count": with_inst(n_real=int(h.n_real) + 1),
    }
    for what, b in bad.items():
        assert load(b) == P.SPH_E_INVALID, what
