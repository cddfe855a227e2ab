"""The C++ host interface (mysph_gb300/host/mysph.hpp): a compiled driver
calls BGGS, con_density, divergence, internal_force, single_step and
time_integration with the reference's names and particle type; its results
match the oracle like the Python path's."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mysph_gb300 import cases
from oracle.oracle import Oracle
from tests.conftest import rel_l2
from tests.helpers import perturb

ROOT = Path(__file__).resolve().parents[1]


def _compile(tmp: Path) -> Path:
    exe = tmp / "host_parity"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"),
                    str(ROOT / "mysph_gb300" / "host" / "mysph.cpp"), str(ROOT / "tests" / "cpp" / "host_parity.cpp"),
                    "-L", str(ROOT / "mysph_gb300"), "-lsphgpu", f"-Wl,-rpath,{ROOT / 'mysph_gb300'}",
                    "-o", str(exe)], check=True)
    return exe


def test_host_interface_compiles(tmp_path):
    from mysph_gb300 import _lib
    _lib.load()                      # the library the driver links
    assert _compile(tmp_path).exists()


def _write_case(path: Path, c) -> None:
    import ctypes
    x, v, m, rho, p, e, cc, h, t, s, b, _ = c.arrays()
    with open(path, "wb") as f:
        f.write(np.array([c.dim, c.n_real, c.n_wall, ctypes.sizeof(c.params)], dtype=np.int32).tobytes())
        f.write(bytes(c.params))
        for a in (x, v, m, rho, p, e, cc, h):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        for a in (t, s, b):
            f.write(np.ascontiguousarray(a, dtype=np.int32).tobytes())


@pytest.mark.gpu
def test_cpp_host_matches_oracle(gpu, tmp_path):
    c = perturb(cases.dam_break_2d(dx=0.05), seed=61, v_amp=0.3, x_frac=0.2)
    _write_case(tmp_path / "case.bin", c)
    exe = _compile(tmp_path)
    steps = 10
    r = subprocess.run([str(exe), str(tmp_path / "case.bin"), str(tmp_path / "out.bin"), str(steps)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Statistics" in r.stdout
    nr, dim = c.n_real, c.dim
    raw = (tmp_path / "out.bin").read_bytes()
    total = np.frombuffer(raw[:8], dtype=np.int64)[0]
    nn = np.frombuffer(raw[8:8 + 4 * nr], dtype=np.int32)
    rest = np.frombuffer(raw[8 + 4 * nr:], dtype=np.float64)
    sizes = [nr, nr, nr, nr * dim, nr * dim, nr, nr, nr * dim, nr * dim, nr, 1, 1]
    parts = np.split(rest, np.cumsum(sizes)[:-1])
    drho, divx, divv, a_in, dvdt, ddrho, dde, x, v, rho, mx, mean = parts
    o = Oracle(c)
    o.bggs()
    off, _ = o.neighbors()
    assert np.array_equal(nn, np.diff(off)) and total == off[-1]
    o.rates()
    for got, key in ((drho, "DRHODT"), (divx, "DIVX"), (divv, "DIVV"), (a_in, "IN_DVDT"), (dvdt, "DVDT"),
                     (ddrho, "DRHODT"), (dde, "DEDT")):
        assert rel_l2(got, o.field(key)[:nr]) <= 1e-10, key
    omx, omean = o.advance(steps)
    for got, key in ((x, "X"), (v, "V"), (rho, "RHO")):
        assert rel_l2(got, o.field(key)[:nr]) <= 1e-8, key
    assert mx[0] == pytest.approx(omx, rel=1e-8) and mean[0] == pytest.approx(omean, rel=1e-8)
