"""The C ABI: the library loads, exports every entry point declared in
include/sph_gpu.h, and the ctypes mirror of sph_params matches the C layout.
No device work is done here (no GPU in this test)."""
import ctypes as C
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from mysph_gb300 import _lib
from mysph_gb300 import params as P

ROOT = Path(__file__).resolve().parents[1]


def test_library_exports_header():
    lib = _lib.load()
    syms = _lib.header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) <= set(_lib.SIGNATURES), set(syms) - set(_lib.SIGNATURES)
    assert lib.sph_abi_version() == 1


def test_params_layout_matches_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "sph_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(sph_params), sizeof(sph_material),
         offsetof(sph_params, materials), offsetof(sph_params, cell_size),
         offsetof(sph_params, grid_margin), offsetof(sph_material, mg_s),
         offsetof(sph_params, xsph_eps));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = Path(d) / "probe.c"
        c.write_text(src)
        exe = Path(d) / "probe"
        subprocess.run(["gcc", "-I", str(ROOT / "include"), str(c), "-o", str(exe)], check=True)
        vals = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    want = [C.sizeof(P.SphParams), C.sizeof(P.SphMaterial), P.SphParams.materials.offset,
            P.SphParams.cell_size.offset, P.SphParams.grid_margin.offset, P.SphMaterial.mg_s.offset,
            P.SphParams.xsph_eps.offset]
    assert vals == want


def test_block_layout_matches_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "sph_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(sph_block), offsetof(sph_block, origin),
         offsetof(sph_block, p_rho0_g), offsetof(sph_block, tait_rho0), offsetof(sph_block, v_ramp_len),
         offsetof(sph_block, clamp_below), offsetof(sph_block, clamp_axis), offsetof(sph_block, clamp_above));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = Path(d) / "probe.c"
        c.write_text(src)
        exe = Path(d) / "probe"
        subprocess.run(["gcc", "-I", str(ROOT / "include"), str(c), "-o", str(exe)], check=True)
        vals = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    B = P.SphBlock
    assert vals == [C.sizeof(B), B.origin.offset, B.p_rho0_g.offset, B.tait_rho0.offset, B.v_ramp_len.offset,
                    B.clamp_below.offset, B.clamp_axis.offset, B.clamp_above.offset]


def _emulate_blocks(bc):
    """The lattice rule of sph_block (include/sph_gpu.h) in numpy: positions,
    hydrostatic pressure, types and the clamp flag, in generation order."""
    dim = bc.dim
    xs, ps, ts, cl = [], [], [], []
    for B in bc.blocks:
        n = [B.n[a] if a < dim else 1 for a in range(3)]
        idx = np.stack(np.meshgrid(*[np.arange(k) for k in n], indexing="ij"), -1).reshape(-1, 3)
        x = np.stack([B.origin[a] + (idx[:, a] + 0.5) * B.spacing[a] for a in range(dim)], 1)
        p = B.p_rho0_g * np.maximum(B.p_level - x[:, B.up_axis], 0.0) if B.p_rho0_g != 0 else np.zeros(len(x))
        xc = x[:, B.clamp_axis]
        xs.append(x); ps.append(p); ts.append(np.full(len(x), B.type))
        cl.append(((xc < B.clamp_below) | (xc > B.clamp_above)).astype(np.int32))
    return np.concatenate(xs), np.concatenate(ps), np.concatenate(ts), np.concatenate(cl)


@pytest.mark.parametrize("name", ["dam2d", "dam3d", "cantilever", "gate"])
def test_block_cases_match_host_cases(name):
    """Each block description generates the host case's lattice: the same
    counts, positions bit for bit, pressures, types and clamped particles."""
    from mysph_gb300 import cases
    bc, hc = {
        "dam2d": lambda: (cases.dam_break_2d_blocks(dx=0.05), cases.dam_break_2d(dx=0.05)),
        "dam3d": lambda: (cases.dam_break_3d_blocks(dx=0.03), cases.dam_break_3d(dx=0.03)),
        "cantilever": lambda: (cases.cantilever_2d_blocks(dx=2e-3, length=0.04, thickness=0.01),
                               cases.cantilever_2d(dx=2e-3, length=0.04, thickness=0.01)),
        "gate": lambda: (cases.gate_2d_blocks(dx=0.0025), cases.gate_2d(dx=0.0025)),
    }[name]()
    assert bc.counts() == (hc.n_real, hc.n_wall)
    assert bc.params.dt == hc.params.dt and bc.params.flags == hc.params.flags
    x, p, t, clamp = _emulate_blocks(bc)
    assert np.array_equal(x, hc.x)
    assert np.allclose(p, hc.p, rtol=0, atol=1e-9 * max(1.0, np.abs(hc.p).max()))
    assert np.array_equal(t, hc.type)
    bnd = np.zeros(len(x), np.int32) if hc.boundary is None else hc.boundary
    assert np.array_equal(clamp[: hc.n_real], bnd[: hc.n_real])


def test_params_default_matches_python():
    lib = _lib.load()
    p = P.SphParams()
    assert lib.sph_params_default(C.byref(p)) == 0
    q = P.base_params(2, 5e-4)
    for name in ("av_alpha", "av_beta", "av_psi", "wall_fs", "wall_r0", "pen_factor",
                 "contact_delta", "as_eps", "xsph_eps", "gravity", "flags", "skf", "pa_sph"):
        assert getattr(p, name) == getattr(q, name), name


def test_create_rejects_bad_params_without_gpu_work():
    lib = _lib.load()
    ctx = C.c_void_p()
    p = P.base_params(2, 1e-4)
    p.dim = 7
    assert lib.sph_create(C.byref(p), 100, C.byref(ctx)) == P.SPH_E_UNSUPPORTED
    p.dim = 2
    p.dt = -1.0
    p.flags = 0
    assert lib.sph_create(C.byref(p), 100, C.byref(ctx)) == P.SPH_E_INVALID
    assert lib.sph_create(None, 100, C.byref(ctx)) == P.SPH_E_INVALID
    assert not ctx.value


def _scope_case(prec=P.PREC_FP64, flags=0, skf=1, sph=2, sle=0):
    p = P.base_params(3, 1e-4)
    p.precision, p.skf, p.pa_sph, p.sle = prec, skf, sph, sle
    p.flags |= flags
    return p


@pytest.mark.parametrize("name,prm", [
    ("df64 + kernel correction", lambda: _scope_case(P.PREC_DF64, P.F_KERNEL_CORRECTION)),
    ("df64 + artificial stress", lambda: _scope_case(P.PREC_DF64, P.F_ARTI_STRESS)),
    ("df64 + Gauss kernel", lambda: _scope_case(P.PREC_DF64, skf=2)),
    ("df64 + quintic kernel", lambda: _scope_case(P.PREC_DF64, skf=3)),
    ("mixed + kernel correction", lambda: _scope_case(P.PREC_MIXED, P.F_KERNEL_CORRECTION)),
    ("SPH = 1 in mixed", lambda: _scope_case(P.PREC_MIXED, sph=1)),
    ("SPH = 3 in df64", lambda: _scope_case(P.PREC_DF64, sph=3)),
    ("SPH = 3 + kernel correction", lambda: _scope_case(flags=P.F_KERNEL_CORRECTION, sph=3)),
    ("SPH = 4", lambda: _scope_case(sph=4)),
    ("SLE = 3", lambda: _scope_case(sle=3)),
    ("artificial heat in mixed", lambda: _scope_case(P.PREC_MIXED, P.F_ARTI_HEAT)),
    ("artificial heat in df64", lambda: _scope_case(P.PREC_DF64, P.F_ARTI_HEAT)),
    ("artificial heat under SPH = 1", lambda: _scope_case(flags=P.F_ARTI_HEAT, sph=1)),
    ("artificial heat + kernel correction", lambda: _scope_case(flags=P.F_ARTI_HEAT | P.F_KERNEL_CORRECTION)),
])
def test_option_scope_is_checked_before_gpu_work(name, prm):
    """The options the GPU path does not implement are refused by
    sph_create with SPH_E_UNSUPPORTED before any device call (so this runs
    without a GPU)."""
    lib = _lib.load()
    ctx = C.c_void_p()
    assert lib.sph_create(C.byref(prm()), 100, C.byref(ctx)) == P.SPH_E_UNSUPPORTED, name
    assert not ctx.value


def test_null_context_is_an_error():
    lib = _lib.load()
    assert lib.sph_single_step(None) == P.SPH_E_INVALID
    assert lib.sph_destroy(None) == P.SPH_E_INVALID
    assert lib.sph_sort_scratch_bytes(-1, 8) == -1
